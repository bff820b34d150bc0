"""The package's vectorised constraint-step energy (used by bench.py's NVE drift
report) against the per-pair loop of the test helper, on reference states (no GPU)."""
import numpy as np
import pytest

from sdmd_gb300.energy import constraint_energy, nve_drift
from sdmd_gb300.system import from_fixture
from tests.energy import constraint_energy as loop_constraint_energy


@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt", "ala10_cyl"])
@pytest.mark.parametrize("stage", [None, "final"])
def test_vectorised_constraint_energy_equals_the_loop(golden, case, stage):
    d = golden(case)
    s = from_fixture(d, "pre", dynamic_stage=stage)
    assert constraint_energy(s) == pytest.approx(loop_constraint_energy(s), rel=1e-12, abs=1e-12)


def test_drift_normalisation():
    assert nve_drift(10.0, 10.5, 100, 0.5, 2e6) == pytest.approx(0.5 / 50 / 2)
