"""The precision sweep (tests/precision_sweep.py) on a small dam-break: every
mode within the parity bar of the FP64 oracle, mass exact, and the modes'
energies close to the FP64 run after a few coupled steps."""
from __future__ import annotations

import pytest

from coupledwateranimation_gb300 import scenes

from _helpers import small_muller
from precision_sweep import sweep

pytestmark = pytest.mark.gpu


def test_precision_sweep_small(lib, orc):
    wl = scenes.Workload("small dam-break", [small_muller((20, 20, 20), 0.02, (128, 128), seed=21, zsub=2)], 8)
    rows = sweep(steps=8, warm=5, workload=wl)
    modes = {r["mode"]: r for r in rows if "mode" in r}
    assert set(modes) == {"fp32", "fp32-cascaded-two-sum", "fp64"}
    for r in modes.values():
        assert r["rho_max_rel"] <= 1e-5
        assert r["p_normwise"] <= 1e-5
        assert max(r["force_normwise"]) <= 1e-5
        assert r["mass_change"] == 0.0
        assert r["ms_per_step"] > 0
        assert r["kinetic_vs_fp64"] <= 1e-3
    assert modes["fp64"]["rho_max_rel"] <= modes["fp32"]["rho_max_rel"]
    assert modes["fp64"]["rho_hist_l1_vs_fp64"] == 0.0
