"""The benchmark workloads built with the oracle's own scene generators.

TEST INFRASTRUCTURE ONLY, like the rest of oracle/: bench.py's CPU legs (the
reference arm and the CPU baseline) build their inputs here, so timing the
CPU restatement loads nothing but oracle/_build/libcwa_oracle.so.  The
generators (orc_scene_defaults, orc_make_dam_break, orc_make_bumps,
orc_make_reference_cube) are independent restatements of the library's, and
tests/test_oracle.py checks that both produce the same bytes, scene by scene
and workload by workload.

The scene description is the ABI's cwa_scene_desc (include/cwa.h), mirrored
here as a ctypes structure (tests/test_oracle.py checks the layout against
the library's mirror).  Workload sizes, seeds and draws follow the five
benchmark workloads: dam-break blocks of Mueller SPH over a Gaussian-bump
height field (configs 0-2), and batches of independent scenes with
log-uniform particle counts (configs 3-4).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import oracle as orc

BASE_SEED = 12345
BUMP_SEED = 1_000_003
PRESET_REFERENCE_3D, PRESET_MULLER = 0, 1


class SceneDesc(C.Structure):
    """cwa_scene_desc (include/cwa.h)."""
    _fields_ = [
        ("preset", C.c_int32), ("n_particles", C.c_int32), ("wave_nx", C.c_int32),
        ("wave_nz", C.c_int32), ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3),
        ("cell_size", C.c_float), ("cell_size_z", C.c_float), ("mass", C.c_float), ("smoothing_length", C.c_float),
        ("visc", C.c_float), ("rest_rho", C.c_float), ("gas_const", C.c_float), ("dt", C.c_float),
        ("gravity", C.c_float * 3), ("wall_restitution", C.c_float),
        ("velocity_damping", C.c_float), ("particle_radius", C.c_float),
        ("crest_height", C.c_float), ("foam_speed", C.c_float), ("wave_lambda", C.c_float),
        ("wave_atten", C.c_float), ("wave_beta", C.c_float), ("wave_mode", C.c_float),
        ("wave_uv_scale", C.c_float * 2), ("wave_uv_offset", C.c_float * 2),
        ("surface_y0", C.c_float), ("surface_restitution", C.c_float), ("couple_gain", C.c_float),
        ("deposit_shift", C.c_int32), ("flags", C.c_int32),
    ]


@dataclass
class Scene:
    desc: SceneDesc
    particles: np.ndarray  # (n, 16) float32: the 64-byte records
    wave: np.ndarray       # (nz, nx) float32 initial u^n = u^(n-1)


@dataclass
class Workload:
    name: str
    scenes: list
    steps: int

    @property
    def n_particles(self) -> int:
        return sum(s.desc.n_particles for s in self.scenes)

    @property
    def n_wave_cells(self) -> int:
        return sum(s.desc.wave_nx * s.desc.wave_nz for s in self.scenes)


def dam_break(lattice, spacing, wave, box_hi=(1.0, 1.0, 1.0), seed=BASE_SEED, n_bumps=8, jitter=0.05,
              zsub=1) -> Scene:
    d = orc.scene_defaults(PRESET_MULLER, spacing, SceneDesc)
    d.cell_size_z = d.cell_size / zsub
    for a in range(3):
        d.box_hi[a] = box_hi[a]
    orc.scene_set_wave_grid(d, wave[0], wave[1])
    n = int(np.prod(lattice))
    d.n_particles = n
    p = orc.make_dam_break(d, lattice, spacing, jitter, seed, n)
    u = orc.make_bumps(d, n_bumps, seed + BUMP_SEED, wave[0], wave[1])
    return Scene(d, p, u)


def config0(seed=BASE_SEED) -> Workload:
    return Workload("c0: 32^3 particles s=0.02, 256^2 wave", [dam_break((32, 32, 32), 0.02, (256, 256),
                                                                         seed=seed)], 200)


def config1(seed=BASE_SEED) -> Workload:
    # 1,048,576 particles as a 128 x 64 x 128 lattice (the stated "128^3"
    # would hold twice as many)
    return Workload("c1: 1,048,576 particles (128x64x128, s=0.0075), 1024^2 wave",
                    [dam_break((128, 64, 128), 0.0075, (1024, 1024), seed=seed)], 500)


def config2(seed=BASE_SEED) -> Workload:
    return Workload("c2: 256x128x128 particles s=0.004, 2048^2 wave",
                    [dam_break((256, 128, 128), 0.004, (2048, 2048), box_hi=(1.024, 1.0, 1.0), seed=seed)], 100)


def _batched(name, n_scenes, n_lo, n_hi, waves, steps, seed) -> Workload:
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        target = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        aspect = float(rng.uniform(0.5, 2.0))
        fill = float(rng.uniform(0.2, 0.5))
        w = int(waves[rng.integers(len(waves))])
        block = np.array([aspect, 1.0, 1.0]) * fill ** (1.0 / 3.0)
        s = float((np.prod(block) / target) ** (1.0 / 3.0))
        dims = np.maximum(1, np.round(block / s)).astype(int)
        out.append(dam_break(tuple(int(x) for x in dims), s, (w, w), box_hi=(aspect, 1.0, 1.0), seed=seed + k))
    return Workload(name, out, steps)


def config3(seed=BASE_SEED, n_scenes=256) -> Workload:
    return _batched("c3: 256 batched small scenes", n_scenes, 2048, 65536, (64, 128, 256, 512), 200, seed)


def config4(seed=BASE_SEED, n_scenes=64) -> Workload:
    return _batched("c4: 64 batched large scenes", n_scenes, 65536, 1048576, (512, 1024, 2048), 100, seed)


def reference_preset() -> Scene:
    """The reference app's own scene: 20,480 particles on its 64 x 5 x 64
    cube, 64^2 wave from InitWave, the shaders' constants."""
    d = orc.scene_defaults(PRESET_REFERENCE_3D, 0.0, SceneDesc)
    p = orc.make_reference_cube(d, d.n_particles)
    return Scene(d, p, orc.wave_init_f32(d))


CONFIGS = {0: config0, 1: config1, 2: config2, 3: config3, 4: config4}


def with_zsub(wl: Workload, zsub: int) -> Workload:
    for s in wl.scenes:
        s.desc.cell_size_z = s.desc.cell_size / zsub
    return wl
