"""Python mirror of the PBD box collisions (cwa_pbd_* in include/cwa.h): the
reference's GridTestPbdGpu3D demo on the uniform grid, deterministic."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import PBD_BOX_DTYPE, PbdParams
from .sim import check


def pbd_defaults() -> PbdParams:
    """The demo's settings: 4096 boxes, 16^3 cells over [-1, 1]^3, dt 0.02."""
    p = PbdParams()
    check(_abi.load().cwa_pbd_defaults(C.byref(p)), "cwa_pbd_defaults")
    return p


def make_boxes(params: PbdParams, seed: int = 12345) -> np.ndarray:
    out = np.zeros(params.n_boxes, PBD_BOX_DTYPE)
    check(_abi.load().cwa_pbd_make_boxes(C.byref(params), seed, out.ctypes.data, len(out)), "cwa_pbd_make_boxes")
    return out


class PbdSim:
    def __init__(self, params: PbdParams | None = None, device: int = 0):
        self._lib = _abi.load()
        self.params = pbd_defaults() if params is None else params
        h = C.c_void_p()
        check(self._lib.cwa_pbd_create(C.byref(self.params), device, C.byref(h)), "cwa_pbd_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            check(self._lib.cwa_pbd_destroy(self._h), "cwa_pbd_destroy")
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

    def upload(self, boxes: np.ndarray) -> None:
        a = np.ascontiguousarray(boxes, dtype=PBD_BOX_DTYPE)
        check(self._lib.cwa_pbd_upload(self._h, a.ctypes.data, len(a)), "cwa_pbd_upload")

    def download(self) -> np.ndarray:
        out = np.zeros(self.params.n_boxes, PBD_BOX_DTYPE)
        check(self._lib.cwa_pbd_download(self._h, out.ctypes.data, len(out)), "cwa_pbd_download")
        return out

    def step(self, n: int = 1) -> None:
        check(self._lib.cwa_pbd_step(self._h, int(n)), "cwa_pbd_step")

    def pair_count(self) -> int:
        v = C.c_int64()
        check(self._lib.cwa_pbd_pair_count(self._h, C.byref(v)), "cwa_pbd_pair_count")
        return v.value
