"""Shared helpers for the GPU parity tests."""
from __future__ import annotations

import numpy as np

from coupledwateranimation_gb300 import Sim, scenes


def records_f32(particles: np.ndarray) -> np.ndarray:
    """64-byte records -> (n, 16) float32 view copy."""
    return np.ascontiguousarray(particles).view(np.float32).reshape(-1, 16).copy()


def load_scene(sim: Sim, k: int, sc: scenes.Scene) -> None:
    sim.upload_particles(k, sc.particles)
    if sc.wave is None:
        sim.wave_reinit(k)
    else:
        sim.upload_wave(k, sc.wave, sc.wave)


def rel_inf(got: np.ndarray, want: np.ndarray) -> float:
    """Normwise relative error max|got - want| / max|want|."""
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    den = np.abs(want).max()
    return float(np.abs(got - want).max() / (den if den > 0 else 1.0))


def small_muller(lattice=(16, 16, 16), spacing=0.02, wave=(64, 64), seed=11, zsub=1, skin=0.0) -> scenes.Scene:
    return scenes.dam_break(lattice, spacing, wave, seed=seed, zsub=zsub, skin=skin)


def small_reference(n: int = 5120) -> scenes.Scene:
    s = scenes.reference()
    s.desc.n_particles = n
    s.particles = s.particles[:n].copy()
    return s


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, np.float32).view(np.uint32)
