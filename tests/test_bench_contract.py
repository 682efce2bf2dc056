"""bench.py's measurement plumbing on CPU: the timed step numbers, the
algorithmic bytes and flops the roofline uses (the per-unit figures of the
measurement contract: 348 B a particle-step, 28 B a grid-cell-step, 20 B a
wave-cell-step), the committed ncu traffic the `roofline.traffic` field
reads, and the HBM peak it divides by."""
from __future__ import annotations

import importlib.util
import json
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("warmup,k,last", [(5, 20, 500), (3, 2, 500), (3, 5, 200), (5, 1, 500), (0, 7, 7)])
def test_timed_steps_spread_over_the_workload(bench, warmup, k, last):
    steps = bench._timed_steps(warmup, k, last)
    assert len(steps) == k and steps == sorted(set(steps))
    assert steps[-1] == last and steps[0] >= warmup + 1
    if k > 1:
        assert steps[0] == warmup + 1
        gaps = [b - a for a, b in zip(steps, steps[1:])]
        assert max(gaps) - min(gaps) <= 1  # evenly spaced


def test_algorithmic_bytes_follow_the_contract(bench):
    # hash + count 20, reorder 140, rho_pres 24, force 64, integrate + coupling 100: 348 B a
    # particle-step; the hash and count ride with integrate (the next step's keys)
    assert sum(bench.BYTES_PER_PARTICLE.values()) == 348
    assert bench.BYTES_PER_PARTICLE == {"grid": 140, "rho_pres": 24, "force": 64, "integrate": 120}
    assert bench.BYTES_PER_GRID_CELL == {"grid": 28}
    assert bench.BYTES_PER_WAVE_CELL == {"wave": 20}
    # 216 candidates x 7 flop + 33 hits x 10 (density) or x 40 (force)
    assert bench.FLOP_PER_PARTICLE == {"rho_pres": 1842, "force": 2832}


def test_committed_traffic_covers_every_pass(bench):
    """Every pass has a per-launch DRAM figure in profiles/, within a sane
    multiple of its algorithmic bytes at the 1M-particle workload."""
    traffic = bench._profiled_traffic()
    n_p, n_c, n_w = 1_048_576, 1_198_563, 1024 * 1024
    for name in ("grid", "rho_pres", "force", "integrate", "wave"):
        assert name in traffic and traffic[name] > 0, name
        alg = (bench.BYTES_PER_PARTICLE.get(name, 0) * n_p + bench.BYTES_PER_GRID_CELL.get(name, 0) * n_c
               + bench.BYTES_PER_WAVE_CELL.get(name, 0) * n_w)
        assert 0.3 * alg < traffic[name] < 6 * alg, (name, traffic[name], alg)


def test_peak_is_the_measured_copy_bandwidth(bench):
    peak, kind = bench._peaks()
    measured = ROOT / "MEASURED_PEAKS.json"
    if measured.exists():
        assert kind == "measured" and peak == float(json.loads(measured.read_text())["hbm_gbs"])
    else:
        assert kind == "fallback" and peak == bench.FALLBACK_HBM_GBS
