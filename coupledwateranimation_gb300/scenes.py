"""Scene presets and the benchmark workloads as seeded synthetic scenes.

All inputs are synthetic; no dataset is involved.  Seeds: particles of scene
k use base_seed + k, its Gaussian-bump height field base_seed + k + BUMP_SEED.

  reference(): the reference app's own scene (CoupledWaterAnimation/Main.cpp:28-35,
      184-204, 735-794): 20,480 particles on the 64x5x64 lattice, 64x64 wave
      initialised by InitWave (splash), the shaders' constants.
  dam_break(lattice, spacing, wave): Mueller SPH dam-break block in the
      corner of the box, jitter U(-0.05 s, 0.05 s), 8 Gaussian bumps.
  config0..config4: the five benchmark workloads (sizes in CONFIGS).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import PARTICLE_DTYPE, PRESET_MULLER, PRESET_REFERENCE_3D, SceneDesc, check, ptr

BASE_SEED = 12345
BUMP_SEED = 1_000_003


@dataclass
class Scene:
    desc: SceneDesc
    particles: np.ndarray
    wave: np.ndarray | None        # initial u^n = u^(n-1); None -> InitWave on the device
    lattice: tuple[int, int, int] = (0, 0, 0)
    spacing: float = 0.0


@dataclass
class Workload:
    name: str
    scenes: list[Scene]
    steps: int
    notes: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n_particles(self) -> int:
        return sum(s.desc.n_particles for s in self.scenes)

    @property
    def n_wave_cells(self) -> int:
        return sum(s.desc.wave_nx * s.desc.wave_nz for s in self.scenes)


def defaults(preset: int, spacing: float = 0.0) -> SceneDesc:
    d = SceneDesc()
    check(_abi.load().cwa_scene_defaults(preset, spacing, C.byref(d)), "cwa_scene_defaults")
    return d


def set_wave_grid(d: SceneDesc, nx: int, nz: int) -> None:
    check(_abi.load().cwa_scene_set_wave_grid(C.byref(d), nx, nz), "cwa_scene_set_wave_grid")


def reference() -> Scene:
    d = defaults(PRESET_REFERENCE_3D)
    p = np.zeros(d.n_particles, PARTICLE_DTYPE)
    check(_abi.load().cwa_make_reference_cube(C.byref(d), ptr(p), d.n_particles),
          "cwa_make_reference_cube")
    return Scene(d, p, None, (64, 5, 64), 2.0 * 0.85 * 0.005)


def dam_break(lattice=(32, 32, 32), spacing=0.02, wave=(256, 256), box_hi=(1.0, 1.0, 1.0),
              seed=BASE_SEED, n_bumps=8, jitter=0.05, zsub=1, skin=0.0) -> Scene:
    """zsub > 1 sorts by z cells of edge cell / zsub; skin > 0 widens the x/y
    cells to h (1 + skin), as Verlet mode with that skin needs."""
    lib = _abi.load()
    d = defaults(PRESET_MULLER, spacing)
    if skin > 0.0:
        d.cell_size = d.smoothing_length * (1.0 + skin) * (1.0 + 1e-6)  # never rounds below h (1 + skin)
    d.cell_size_z = d.cell_size / zsub
    for a in range(3):
        d.box_hi[a] = box_hi[a]
    set_wave_grid(d, wave[0], wave[1])
    n = int(np.prod(lattice))
    d.n_particles = n
    dims = (C.c_int32 * 3)(*lattice)
    p = np.zeros(n, PARTICLE_DTYPE)
    check(lib.cwa_make_dam_break(C.byref(d), dims, spacing, jitter, seed, ptr(p), n),
          "cwa_make_dam_break")
    u = np.zeros((wave[1], wave[0]), np.float32)
    check(lib.cwa_make_bumps(C.byref(d), n_bumps, seed + BUMP_SEED, ptr(u), wave[0], wave[1]),
          "cwa_make_bumps")
    return Scene(d, p, u, tuple(lattice), spacing)


def config0(seed=BASE_SEED) -> Workload:
    return Workload("c0: 32^3 particles s=0.02, 256^2 wave", [dam_break((32, 32, 32), 0.02, (256, 256),
                                                                         seed=seed)], 200)


def config1(seed=BASE_SEED) -> Workload:
    # The workload is stated as 1,048,576 particles on a "128^3" lattice, which
    # disagree (128^3 = 2,097,152); the particle count is kept: 128 x 64 x 128
    # (x, y, z), a 0.96 x 0.48 x 0.96 block.
    return Workload("c1: 1,048,576 particles (128x64x128, s=0.0075), 1024^2 wave",
                    [dam_break((128, 64, 128), 0.0075, (1024, 1024), seed=seed)], 500,
                    notes="128x64x128 lattice keeps the stated 1,048,576 particles")


def config2(seed=BASE_SEED) -> Workload:
    # 256 x 0.004 = 1.024 exceeds the unit box: the box x extent is 1.024.
    return Workload("c2: 256x128x128 particles s=0.004, 2048^2 wave",
                    [dam_break((256, 128, 128), 0.004, (2048, 2048), box_hi=(1.024, 1.0, 1.0),
                               seed=seed)], 100, notes="box x extent 1.024")


def _batched(name, n_scenes, n_lo, n_hi, waves, steps, seed) -> Workload:
    """Independent scenes: N ~ log-uniform[n_lo, n_hi], box aspect (x) ~ U(0.5, 2),
    dam-break fill fraction ~ U(0.2, 0.5), lattice dims fitted to the block by
    cube root, wave grid drawn uniformly from `waves`."""
    rng = np.random.default_rng(seed)
    scenes = []
    for k in range(n_scenes):
        target = float(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        aspect = float(rng.uniform(0.5, 2.0))
        fill = float(rng.uniform(0.2, 0.5))
        w = int(waves[rng.integers(len(waves))])
        block = np.array([aspect, 1.0, 1.0]) * fill ** (1.0 / 3.0)
        s = float((np.prod(block) / target) ** (1.0 / 3.0))
        dims = np.maximum(1, np.round(block / s)).astype(int)
        scenes.append(dam_break(tuple(int(x) for x in dims), s, (w, w), box_hi=(aspect, 1.0, 1.0),
                                seed=seed + k))
    return Workload(name, scenes, steps)


def config3(seed=BASE_SEED, n_scenes=256) -> Workload:
    return _batched("c3: 256 batched small scenes", n_scenes, 2048, 65536, (64, 128, 256, 512), 200,
                    seed)


def config4(seed=BASE_SEED, n_scenes=64) -> Workload:
    return _batched("c4: 64 batched large scenes", n_scenes, 65536, 1048576, (512, 1024, 2048), 100,
                    seed)


CONFIGS = {0: config0, 1: config1, 2: config2, 3: config3, 4: config4}


def with_zsub(wl: Workload, zsub: int) -> Workload:
    """The same workload with the sort grid's z cells split zsub times."""
    for s in wl.scenes:
        s.desc.cell_size_z = s.desc.cell_size / zsub
    return wl


def with_grid(wl: Workload, zsub: int = 1, skin: float = 0.0) -> Workload:
    """The same workload with x/y cells of h (1 + skin) (as Verlet mode with
    that skin needs) and z cells of that edge / zsub."""
    for s in wl.scenes:
        if skin > 0.0:
            s.desc.cell_size = s.desc.smoothing_length * (1.0 + skin) * (1.0 + 1e-6)
        s.desc.cell_size_z = s.desc.cell_size / zsub
    return wl
