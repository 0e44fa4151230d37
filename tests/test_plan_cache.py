"""The function-level API's plan cache (sarsolver_gb300.cxx_binding) keys plans on the geometry's
content, never on object identity: a freed aperture's id can be reused by a new one, and an
aperture can be changed in place (e.g. a new slow-time weighting), and neither may reuse a plan
built for other device tables.  CPU only: the plan class is replaced by a recorder."""
import gc

import numpy as np
import pytest

from cases import spotlight_case
from sarsolver_gb300 import cxx_binding


class FakePlan:
    made = []

    def __init__(self, scene, aperture, upsample_ratio, interp):
        self.weights = np.array(aperture.slow_time_weighting, copy=True)
        FakePlan.made.append(self)


@pytest.fixture(autouse=True)
def fake_plans(monkeypatch):
    FakePlan.made = []
    cxx_binding._PLAN_CACHE.clear()
    monkeypatch.setattr(cxx_binding, "SarPlan", FakePlan)
    yield
    cxx_binding._PLAN_CACHE.clear()


def test_same_content_shares_a_plan():
    a = spotlight_case(16, 64, 32, 0.5, 3.0)
    b = spotlight_case(16, 64, 32, 0.5, 3.0)   # equal content, different objects
    p1 = cxx_binding._plan_for(a.scene, a.aperture, 8.0, "linear")
    p2 = cxx_binding._plan_for(b.scene, b.aperture, 8.0, "linear")
    assert p1 is p2 and len(FakePlan.made) == 1
    assert cxx_binding._plan_for(a.scene, a.aperture, 8.0, "nearest_ref") is not p1
    assert cxx_binding._plan_for(a.scene, a.aperture, 16.0, "linear") is not p1


def test_new_aperture_after_freeing_the_old_one_gets_a_new_plan():
    a = spotlight_case(16, 64, 32, 0.5, 3.0)
    p1 = cxx_binding._plan_for(a.scene, a.aperture, 8.0, "linear")
    del a
    gc.collect()
    b = spotlight_case(16, 64, 32, 0.5, 5.0)   # another aperture; may land on the freed ids
    p2 = cxx_binding._plan_for(b.scene, b.aperture, 8.0, "linear")
    assert p2 is not p1 and len(FakePlan.made) == 2


def test_weighting_changed_in_place_gets_a_new_plan():
    rng = np.random.default_rng(1)
    a = spotlight_case(16, 64, 32, 0.5, 3.0)
    p1 = cxx_binding._plan_for(a.scene, a.aperture, 8.0, "linear")
    w = np.exp(1j * rng.uniform(-1, 1, 16))
    a.aperture._slow_time_weighting = w
    assert np.allclose(a.aperture.slow_time_weighting, w)
    p2 = cxx_binding._plan_for(a.scene, a.aperture, 8.0, "linear")
    assert p2 is not p1 and np.allclose(p2.weights, w)


def test_cache_is_bounded():
    for k in range(12):
        c = spotlight_case(8, 32, 32, 0.5, 2.0 + 0.1 * k)
        cxx_binding._plan_for(c.scene, c.aperture, 8.0, "linear")
    assert len(cxx_binding._PLAN_CACHE) <= cxx_binding._PLAN_CACHE_SIZE
