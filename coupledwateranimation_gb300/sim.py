"""Host-side mirror of the reference's step interface over the C ABI.

The reference drives its step from idle() (CoupledWaterAnimation/Main.cpp:530-562):
three particle dispatches (rho_pres, force, integrate) and Module::sComputeAll(),
which runs StencilImage2DTripleBuffered::Compute (the wave evolve + PingPong).
`Sim` exposes the same passes one by one (`rho_pres`, `force`, `integrate`,
`wave`, plus the grid sort that precedes them) and the whole step (`step`).
`WaveModule` mirrors the Module hooks Init / Reinit / Compute of
StencilImage2DTripleBuffered (StencilImage2DTripleBuffered.h:8-41).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import (PARTICLE_DTYPE, PASSES, PREC_COMPENSATED, TOTALS, DeviceView, SceneDesc,
                   SimOptions, check, ptr)


@dataclass
class GridArrays:
    cell_start: np.ndarray  # n_cells + 1, scene-local offsets
    sorted_id: np.ndarray   # upload index of each sorted particle


def render_defaults(width: int, height: int):
    """(Camera, RenderParams) of the reference's startup view."""
    cam, prm = _abi.Camera(), _abi.RenderParams()
    check(_abi.load().cwa_render_defaults(width, height, C.byref(cam), C.byref(prm)), "cwa_render_defaults")
    return cam, prm


class Sim:
    """One or more independent scenes stepped together on one GPU."""

    def __init__(self, scenes, precision: int = PREC_COMPENSATED, use_graph: bool = True,
                 device: int = 0, nb_threads: int = 0, nb_stage: int = 0, verlet_skin: float = 0.0,
                 nb_scan_minb: int = 0, nb_force_minb: int = 0, wave_block: int = 0, nb_queue: int = 0):
        self._lib = _abi.load()
        if isinstance(scenes, SceneDesc):
            scenes = [scenes]
        self.scenes = [s.copy() for s in scenes]
        arr = (SceneDesc * len(self.scenes))(*self.scenes)
        opt = SimOptions(device=device, precision=precision, use_graph=int(use_graph),
                         nb_threads=nb_threads, nb_stage=nb_stage, verlet_skin=verlet_skin,
                         nb_scan_minb=nb_scan_minb, nb_force_minb=nb_force_minb, wave_block=wave_block,
                         nb_queue=nb_queue)
        h = C.c_void_p()
        check(self._lib.cwa_create(C.byref(opt), arr, len(self.scenes), C.byref(h)), "cwa_create")
        self._h = h

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            check(self._lib.cwa_destroy(self._h), "cwa_destroy")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- data in / out -----------------------------------------------------
    def upload_particles(self, scene: int, particles: np.ndarray) -> None:
        p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
        check(self._lib.cwa_upload_particles(self._h, scene, ptr(p), len(p)), "cwa_upload_particles")

    def download_particles(self, scene: int = 0) -> np.ndarray:
        n = self.scenes[scene].n_particles
        out = np.zeros(n, dtype=PARTICLE_DTYPE)
        check(self._lib.cwa_download_particles(self._h, scene, ptr(out), n), "cwa_download_particles")
        return out

    def upload_wave(self, scene: int, u_n: np.ndarray, u_nm1: np.ndarray | None = None) -> None:
        d = self.scenes[scene]
        a = np.ascontiguousarray(u_n, dtype=np.float32).reshape(d.wave_nz, d.wave_nx)
        b = None if u_nm1 is None else np.ascontiguousarray(u_nm1, dtype=np.float32).reshape(a.shape)
        check(self._lib.cwa_upload_wave(self._h, scene, ptr(a), ptr(b), d.wave_nx, d.wave_nz),
              "cwa_upload_wave")

    def download_wave(self, scene: int = 0) -> tuple[np.ndarray, np.ndarray]:
        d = self.scenes[scene]
        a = np.zeros((d.wave_nz, d.wave_nx), np.float32)
        b = np.zeros_like(a)
        check(self._lib.cwa_download_wave(self._h, scene, ptr(a), ptr(b), d.wave_nx, d.wave_nz),
              "cwa_download_wave")
        return a, b

    def wave_reinit(self, scene: int = 0) -> None:
        check(self._lib.cwa_wave_reinit(self._h, scene), "cwa_wave_reinit")

    # -- the step ------------------------------------------------------------
    def step(self, n: int = 1) -> None:
        check(self._lib.cwa_step(self._h, n), "cwa_step")

    def grid(self) -> None:
        check(self._lib.cwa_pass_grid(self._h), "cwa_pass_grid")

    def rho_pres(self) -> None:
        check(self._lib.cwa_pass_rho_pres(self._h), "cwa_pass_rho_pres")

    def force(self) -> None:
        check(self._lib.cwa_pass_force(self._h), "cwa_pass_force")

    def integrate(self) -> None:
        check(self._lib.cwa_pass_integrate(self._h), "cwa_pass_integrate")

    def wave(self) -> None:
        check(self._lib.cwa_pass_wave(self._h), "cwa_pass_wave")

    def wave_init_from_image(self, scene: int, rgba: np.ndarray) -> None:
        """ReinitFromTexture: u^n <- red(2x, y) / 255 of an (h, w, 4) uint8
        texture whose row 0 is texture row 0; u^(n-1) <- the old u^n."""
        img = np.ascontiguousarray(rgba, dtype=np.uint8)
        if img.ndim != 3 or img.shape[2] != 4:
            raise ValueError("expected an (h, w, 4) RGBA8 image")
        check(self._lib.cwa_wave_init_from_image(self._h, scene, img.ctypes.data, img.shape[1], img.shape[0]),
              "cwa_wave_init_from_image")

    def set_skybox(self, faces: np.ndarray) -> None:
        """Environment cube map: (6, S, S, 4) uint8 faces +x, -x, +y, -y, +z, -z,
        rows top-down as stored in the image files."""
        f = np.ascontiguousarray(faces, dtype=np.uint8)
        if f.ndim != 4 or f.shape[0] != 6 or f.shape[1] != f.shape[2] or f.shape[3] != 4:
            raise ValueError("expected (6, S, S, 4) RGBA8 faces")
        check(self._lib.cwa_render_set_skybox(self._h, f.ctypes.data, f.shape[1]), "cwa_render_set_skybox")

    def render(self, scene: int = 0, width: int = 640, height: int = 360, camera=None, params=None,
               **overrides) -> np.ndarray:
        """One headless frame as an (height, width, 4) uint8 image, row 0 at the
        bottom (glReadPixels order).  `camera` / `params` default to the
        reference's startup view; keyword overrides set RenderParams fields
        (angle, particle_scale, wave_scale, point_size, surface_res,
        draw_surface, draw_particles, draw_skybox)."""
        cam, prm = render_defaults(width, height)
        if camera is not None:
            cam = camera
        if params is not None:
            prm = params
        for k, v in overrides.items():
            setattr(prm, k, v)
        out = np.zeros((prm.height, prm.width, 4), np.uint8)
        check(self._lib.cwa_render(self._h, scene, C.byref(cam), C.byref(prm), out.ctypes.data), "cwa_render")
        return out

    def wave_advance(self, n: int) -> None:
        """n wave passes with no particle passes between them (K per launch,
        K from the wave_block option)."""
        check(self._lib.cwa_wave_advance(self._h, int(n)), "cwa_wave_advance")

    def synchronize(self) -> None:
        check(self._lib.cwa_synchronize(self._h), "cwa_synchronize")

    # -- inspection ----------------------------------------------------------
    @property
    def step_count(self) -> int:
        v = C.c_int64()
        check(self._lib.cwa_get_step_count(self._h, C.byref(v)), "cwa_get_step_count")
        return v.value

    @property
    def rebuild_count(self) -> int:
        v = C.c_int64()
        check(self._lib.cwa_get_rebuild_count(self._h, C.byref(v)), "cwa_get_rebuild_count")
        return v.value

    @property
    def launch_count(self) -> int:
        v = C.c_int64()
        check(self._lib.cwa_get_launch_count(self._h, C.byref(v)), "cwa_get_launch_count")
        return v.value

    def grid_dims(self, scene: int = 0) -> tuple[int, int, int]:
        dims = (C.c_int32 * 3)()
        check(self._lib.cwa_grid_dims(C.byref(self.scenes[scene]), dims), "cwa_grid_dims")
        return tuple(dims)

    def download_grid(self, scene: int = 0) -> GridArrays:
        d = self.scenes[scene]
        nc = int(np.prod(self.grid_dims(scene)))
        start = np.zeros(nc + 1, np.int32)
        sid = np.zeros(d.n_particles, np.int32)
        check(self._lib.cwa_download_grid(self._h, scene, ptr(start), nc + 1, ptr(sid), d.n_particles),
              "cwa_download_grid")
        return GridArrays(start, sid)

    def download_deposits(self, scene: int = 0) -> np.ndarray:
        d = self.scenes[scene]
        out = np.zeros((d.wave_nz, d.wave_nx), np.int64)
        check(self._lib.cwa_download_deposits(self._h, scene, ptr(out), d.wave_nx, d.wave_nz),
              "cwa_download_deposits")
        return out

    def totals(self, scene: int = 0) -> dict[str, float]:
        out = np.zeros(len(TOTALS), np.float64)
        check(self._lib.cwa_reduce_totals(self._h, scene, ptr(out)), "cwa_reduce_totals")
        return dict(zip(TOTALS, out.tolist()))

    def device_view(self, scene: int = 0) -> DeviceView:
        v = DeviceView()
        check(self._lib.cwa_get_device_view(self._h, scene, C.byref(v)), "cwa_get_device_view")
        return v

    def save(self, path: str) -> None:
        check(self._lib.cwa_save(self._h, str(path).encode()), "cwa_save")

    def load(self, path: str) -> None:
        check(self._lib.cwa_load(self._h, str(path).encode()), "cwa_load")

    def autotune(self, trial_steps: int = 5) -> dict:
        """Pick the fastest neighbour-pass kernel variants for this sim's state
        (see cwa_autotune); the state is restored afterwards."""
        r = _abi.TuneReport()
        check(self._lib.cwa_autotune(self._h, trial_steps, C.byref(r)), "cwa_autotune")
        opt = lambda o: {"nb_stage": o.nb_stage, "nb_scan_minb": o.nb_scan_minb,  # noqa: E731
                         "nb_force_minb": o.nb_force_minb, "nb_threads": o.nb_threads}
        n = min(r.n_tried, 32)
        return {"best": opt(r.best), "best_ms": r.best_ms, "entry_ms": r.entry_ms,
                "tried": [dict(opt(r.tried[k]), ms=r.tried_ms[k]) for k in range(n)]}

    def autotune_wave(self, trial_steps: int = 64) -> dict:
        """Pick the fastest blocked wave-advance variant for this sim's wave
        state (see cwa_autotune_wave); the state is restored afterwards."""
        r = _abi.WaveTuneReport()
        check(self._lib.cwa_autotune_wave(self._h, trial_steps, C.byref(r)), "cwa_autotune_wave")
        return {"best": r.best, "best_name": _abi.WAVE_BLOCKS[r.best], "steps": r.steps,
                "ms_per_step": dict(zip(_abi.WAVE_BLOCKS, list(r.ms_per_step)))}

    def options(self) -> dict:
        o = _abi.SimOptions()
        check(self._lib.cwa_get_options(self._h, C.byref(o)), "cwa_get_options")
        return {f: getattr(o, f) for f, _ in o._fields_ if f != "reserved"}

    def set_profiling(self, on: bool) -> None:
        check(self._lib.cwa_set_profiling(self._h, int(on)), "cwa_set_profiling")

    def pass_times(self) -> dict[str, float]:
        out = np.zeros(len(PASSES), np.float32)
        check(self._lib.cwa_get_pass_times(self._h, ptr(out), len(PASSES)), "cwa_get_pass_times")
        return dict(zip(PASSES, out.tolist()))


class WaveModule:
    """StencilImage2DTripleBuffered's Module hooks over one scene of a Sim.

    Init / Reinit run the MODE_INIT dispatch into both history buffers
    (StencilImage2DTripleBuffered.cpp:10-59); Compute runs one EvolveWave +
    PingPong (:79-95).  GetReadImage(0/1) return u^n and u^(n-1).
    """

    def __init__(self, sim: Sim, scene: int = 0):
        self.sim, self.scene = sim, scene

    def Init(self) -> None:  # noqa: N802 (reference method names)
        self.Reinit()

    def Reinit(self) -> None:  # noqa: N802
        self.sim.wave_reinit(self.scene)

    def Compute(self) -> None:  # noqa: N802
        self.sim.wave()

    def GetReadImage(self, i: int) -> np.ndarray:  # noqa: N802
        return self.sim.download_wave(self.scene)[i]
