"""Python mirror of the 2D solver family (cwa2d_* in include/cwa.h): the
reference's SphWave2D app, cubic-spline SPH with signed-distance walls
driven by a 1D shallow-water field (the app's active choice) or by the 1D
damped wave equation (Wave1D_cs.glsl)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import PARTICLE2D_DTYPE, PASS2D, WAVE2D_1D, WAVE2D_SHALLOW, Params2D
from .sim import check


def defaults2d(wave_kind: int = WAVE2D_SHALLOW) -> Params2D:
    """SphWave2D's own settings: 4096 particles, 32 x 32 grid, and either the
    shallow-water field (128 cells, one substep, lambda 0.001) or, with
    wave_kind=WAVE2D_1D, the app's InitWaveEquation settings (Main.cpp:63-75:
    1024 cells, 10 substeps, three buffers; Wave1D_cs.glsl:21-23 lambda 0.01,
    atten 0.9995, beta 0.001)."""
    p = Params2D()
    check(_abi.load().cwa2d_defaults(C.byref(p)), "cwa2d_defaults")
    if wave_kind == WAVE2D_1D:
        p.wave_kind = WAVE2D_1D
        p.wave_cells = 1024
        p.wave_substeps = 10
        p.wave_lambda = 0.01
    return p


class Sim2D:
    """One SphWave2D scene on one GPU: SphUgrid (two substeps of grid,
    density, forces) followed by the wave substeps, per frame."""

    def __init__(self, params: Params2D | None = None, device: int = 0):
        self._lib = _abi.load()
        self.params = defaults2d() if params is None else params
        h = C.c_void_p()
        check(self._lib.cwa2d_create(C.byref(self.params), device, C.byref(h)), "cwa2d_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            check(self._lib.cwa2d_destroy(self._h), "cwa2d_destroy")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 (interpreter shutdown)
            pass

    def reinit(self) -> None:
        check(self._lib.cwa2d_reinit(self._h), "cwa2d_reinit")

    def splash(self) -> None:
        check(self._lib.cwa2d_splash(self._h), "cwa2d_splash")

    def step(self, n: int = 1) -> None:
        check(self._lib.cwa2d_step(self._h, int(n)), "cwa2d_step")

    def run_pass(self, name: str) -> None:
        check(self._lib.cwa2d_pass(self._h, PASS2D[name]), f"cwa2d_pass({name})")

    def synchronize(self) -> None:
        check(self._lib.cwa2d_synchronize(self._h), "cwa2d_synchronize")

    def upload_particles(self, particles: np.ndarray) -> None:
        a = np.ascontiguousarray(particles, dtype=PARTICLE2D_DTYPE)
        check(self._lib.cwa2d_upload_particles(self._h, a.ctypes.data, len(a)), "cwa2d_upload_particles")

    def download_particles(self) -> np.ndarray:
        out = np.zeros(self.params.n_particles, PARTICLE2D_DTYPE)
        check(self._lib.cwa2d_download_particles(self._h, out.ctypes.data, len(out)), "cwa2d_download_particles")
        return out

    def upload_wave(self, cells4: np.ndarray) -> None:
        a = np.ascontiguousarray(cells4, dtype=np.float32).reshape(-1, 4)
        check(self._lib.cwa2d_upload_wave(self._h, a.ctypes.data, len(a)), "cwa2d_upload_wave")

    def download_wave(self) -> np.ndarray:
        out = np.zeros((self.params.wave_cells, 4), np.float32)
        check(self._lib.cwa2d_download_wave(self._h, out.ctypes.data, len(out)), "cwa2d_download_wave")
        return out

    def upload_wave_prev(self, cells4: np.ndarray) -> None:
        """Wave1D kind: the field one step older than the newest."""
        a = np.ascontiguousarray(cells4, dtype=np.float32).reshape(-1, 4)
        check(self._lib.cwa2d_upload_wave_prev(self._h, a.ctypes.data, len(a)), "cwa2d_upload_wave_prev")

    def download_wave_prev(self) -> np.ndarray:
        out = np.zeros((self.params.wave_cells, 4), np.float32)
        check(self._lib.cwa2d_download_wave_prev(self._h, out.ctypes.data, len(out)), "cwa2d_download_wave_prev")
        return out
