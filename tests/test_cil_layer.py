"""CIL operator layer (src/sarsolver/cil/*.py) without a GPU: geometry shapes, dtypes and
allocation, container semantics, and the choice between real CIL (here a fake of its surface)
and the built-in stand-in."""
import importlib

import numpy as np
import pytest

import fake_cil
from cases import load_golden


@pytest.fixture
def cil_with_fake():
    saved = fake_cil.install()
    import sarsolver_gb300.cil as mod
    mod = importlib.reload(mod)
    yield mod
    fake_cil.uninstall(saved)
    importlib.reload(mod)


@pytest.fixture
def cil_without():
    import sarsolver_gb300.cil as mod
    return importlib.reload(mod)


def test_uses_real_cil_surface_when_present(cil_with_fake):
    mod = cil_with_fake
    assert mod.HAVE_CIL
    assert issubclass(mod.ExtendedDataContainer, fake_cil.DataContainer)
    assert issubclass(mod.GpuCilSarOperator, fake_cil.LinearOperator)
    assert mod.FillType is fake_cil.FillType
    assert mod.CpuSarOperator is mod.GpuCilSarOperator


@pytest.mark.parametrize("use_fake", [True, False])
def test_geometries(use_fake, request):
    mod = request.getfixturevalue("cil_with_fake" if use_fake else "cil_without")
    case = load_golden("little")
    img = mod.CilSarGridGeometry(case.scene)
    meas = mod.SimpleCilSarGeometry(case.aperture)
    assert tuple(img.shape) == tuple(case.scene.grid_shape)          # (z, y, x), cil/hypothesis.py:38-47
    assert list(meas.shape) == [249, 251]                            # [S, N], cil/measurement.py:38-47
    a = img.allocate()
    assert a.array.dtype == np.complex128 and a.array.shape == tuple(img.shape) and not a.array.any()
    assert a.geometry is not img and tuple(a.geometry.shape) == tuple(img.shape)   # deep copy
    r = meas.allocate(mod.FillType.RANDOM, seed=3)
    assert np.iscomplexobj(r.array) and r.array.imag.any()
    r2 = meas.allocate(mod.FillType.RANDOM, seed=3)
    assert np.array_equal(r.array, r2.array)
    i = meas.allocate(mod.FillType.RANDOM_INT, seed=1, max_value=7)
    assert i.array.real.max() < 7 and i.array.dtype == np.complex128
    v = img.allocate(2.5)
    assert np.all(v.array == 2.5)
    img.dtype = np.complex64
    assert img.allocate().array.dtype == np.complex64


def test_fallback_linear_operator_surface(cil_without):
    mod = cil_without
    if mod.HAVE_CIL:
        pytest.skip("real CIL installed")
    case = load_golden("little")
    op = mod.GpuCilSarOperator(mod.CilSarGridGeometry(case.scene), mod.SimpleCilSarGeometry(case.aperture))
    assert op.is_linear()
    assert op.domain is op.domain_geometry() and op.range is op.range_geometry()
