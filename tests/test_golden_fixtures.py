"""The committed oracle trajectory fixtures hold the reference's own
acceptance values for their regression decks (tests/KKScomposition
test3d.py:38-62, tests/SingleGrainGrowthAuNi test2d.py:38-64): the runs
they record are the ones the GPU regression tests compare with."""
import json

import pytest

import kkscomposition as K
import singlegrain as SG


@pytest.mark.parametrize("path,target,tol,drift_tol,diffusivities", [
    (K.FIXTURE, K.SOLID_TARGET, K.SOLID_TOL, K.DRIFT_TOL, "the deck's D_L, D_S"),
    (K.FIXTURE_MOBILITY, K.SOLID_TARGET, K.SOLID_TOL, K.DRIFT_TOL, "atomic mobilities"),
    (SG.FIXTURE, SG.SOLID_TARGET, SG.SOLID_TOL, SG.DRIFT_TOL, None),
])
def test_fixture_meets_acceptance(path, target, tol, drift_tol, diffusivities):
    with open(path) as f:
        gold = json.load(f)
    assert abs(gold["t"][-1] - 0.3) < 1e-9
    assert abs(gold["solid"][-1] - target) <= tol
    assert abs(gold["drift"]) < drift_tol
    assert gold["solid"] == sorted(gold["solid"])  # the grain grows
    if diffusivities is not None:
        assert gold.get("diffusivities", "the deck's D_L, D_S") == diffusivities
