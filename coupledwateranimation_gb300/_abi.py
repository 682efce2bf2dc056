"""ctypes binding of the C ABI in include/cwa.h (libcwa.so, built in-tree).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

# CWA_LIBRARY=debug selects the index-checked build (libcwa_debug.so, made by
# build.build(debug=True)); the default is the release library.
LIB_PATH = Path(__file__).resolve().parent / (
    "libcwa_debug.so" if os.environ.get("CWA_LIBRARY") == "debug" else "libcwa.so")

# status codes
CWA_OK = 0
CWA_ERR_INVALID_ARG = 1
CWA_ERR_OOM = 2
CWA_ERR_CUDA = 3
CWA_ERR_TIMEOUT = 4
CWA_ERR_NONFINITE = 5
CWA_ERR_IO = 6
CWA_ERR_NO_DEVICE = 7
CWA_ERR_CAPACITY = 8
CWA_ERR_BOUNDS = 9

PRESET_REFERENCE_3D = 0
PRESET_MULLER = 1
PREC_FP32, PREC_COMPENSATED, PREC_FP64 = 0, 1, 2

TOTALS = ("mass", "momentum_x", "momentum_y", "momentum_z", "kinetic", "potential", "wave_volume",
          "wave_energy")
PASSES = ("grid", "rho_pres", "force", "integrate", "wave")

# numpy view of cwa_particle (64 bytes, std430 Particle)
PARTICLE_DTYPE = np.dtype([("pos", "<f4", 4), ("vel", "<f4", 4), ("force", "<f4", 4),
                           ("extras", "<f4", 4)])


class SceneDesc(C.Structure):
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

    def copy(self) -> "SceneDesc":
        out = SceneDesc()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(SceneDesc))
        return out


class SimOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("use_graph", C.c_int32),
                ("nb_threads", C.c_int32), ("nb_stage", C.c_int32), ("verlet_skin", C.c_float),
                ("nb_scan_minb", C.c_int32), ("nb_force_minb", C.c_int32), ("wave_block", C.c_int32),
                ("nb_queue", C.c_int32), ("reserved", C.c_int32 * 2)]


# CWA_WAVE_BLOCK_*: box rows x steps per launch; R = box column in registers,
# P = 256-wide box with column pairs in registers, S = persistent register
# form with the next box prefetched
WAVE_BLOCKS = ("32x4", "64x4", "64x8", "R32x4", "R64x4", "R64x8", "P32x4", "S32x4")


class WaveTuneReport(C.Structure):
    _fields_ = [("best", C.c_int32), ("steps", C.c_int32), ("ms_per_step", C.c_float * len(WAVE_BLOCKS))]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("center", C.c_float * 3), ("up", C.c_float * 3), ("fovy", C.c_float),
                ("near_z", C.c_float), ("far_z", C.c_float)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("angle", C.c_float), ("particle_scale", C.c_float),
                ("wave_scale", C.c_float), ("point_size", C.c_float), ("surface_res", C.c_int32),
                ("draw_surface", C.c_int32), ("draw_particles", C.c_int32), ("draw_skybox", C.c_int32),
                ("reserved", C.c_int32 * 4)]


class Params2D(C.Structure):
    _fields_ = [("n_particles", C.c_int32), ("wave_cells", C.c_int32), ("sph_substeps", C.c_int32),
                ("wave_substeps", C.c_int32), ("grid_cells", C.c_int32 * 2), ("init_columns", C.c_int32),
                ("view_size", C.c_float * 2), ("particle_radius", C.c_float), ("rest_density", C.c_float),
                ("visc", C.c_float), ("dt", C.c_float), ("gas_const", C.c_float), ("bottom", C.c_float),
                ("wave_lambda", C.c_float), ("wave_dx", C.c_float), ("wave_kind", C.c_int32),
                ("wave_atten", C.c_float), ("wave_beta", C.c_float), ("reserved", C.c_int32 * 1)]


WAVE2D_SHALLOW, WAVE2D_1D = 0, 1  # CWA2D_WAVE_*


class PbdParams(C.Structure):
    _fields_ = [("n_boxes", C.c_int32), ("grid_cells", C.c_int32 * 3), ("extents_lo", C.c_float * 3),
                ("extents_hi", C.c_float * 3), ("g", C.c_float * 3), ("dt", C.c_float), ("damping", C.c_float),
                ("k", C.c_float), ("k_static", C.c_float), ("sleep_thresh", C.c_float), ("mu_k", C.c_float),
                ("mu_s", C.c_float), ("e", C.c_float), ("substeps", C.c_int32), ("max_contacts", C.c_int32),
                ("reserved", C.c_int32 * 3)]


PBD_BOX_DTYPE = np.dtype([("color", "<f4", 4), ("x", "<f4", 4), ("v", "<f4", 4), ("p", "<f4", 4),
                          ("dp_t", "<f4", 4), ("dp_n", "<f4", 4), ("hw", "<f4", 4), ("rm", "<f4"), ("n", "<f4"),
                          ("e", "<f4"), ("padding", "<f4")])
PARTICLE2D_DTYPE = np.dtype([("pos", "<f4", 4), ("vel", "<f4", 4), ("acc", "<f4", 4)])
PASS2D = {"grid": 0, "density": 1, "force": 2, "wave_predict": 3, "wave_correct": 4, "wave_iterate": 5}


class TuneReport(C.Structure):
    _fields_ = [("best", SimOptions), ("best_ms", C.c_float), ("entry_ms", C.c_float),
                ("n_tried", C.c_int32), ("tried", SimOptions * 32), ("tried_ms", C.c_float * 32)]


class DeviceView(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int32), ("n_cells", C.c_int32), ("grid_dims", C.c_int32 * 3),
        ("wave_nx", C.c_int32), ("wave_nz", C.c_int32), ("pos", C.c_void_p), ("vel", C.c_void_p),
        ("force", C.c_void_p), ("rho_p", C.c_void_p), ("particle_id", C.c_void_p),
        ("cell_start", C.c_void_p), ("wave_u_n", C.c_void_p), ("wave_u_nm1", C.c_void_p),
        ("stream", C.c_void_p),
    ]


_P = C.c_void_p
_I32 = C.c_int32
_PROTOS = {
    "cwa_status_str": (C.c_char_p, [C.c_int]),
    "cwa_abi_version": (_I32, []),
    "cwa_last_error": (C.c_char_p, []),
    "cwa_scene_defaults": (C.c_int, [_I32, C.c_float, C.POINTER(SceneDesc)]),
    "cwa_scene_set_wave_grid": (C.c_int, [C.POINTER(SceneDesc), _I32, _I32]),
    "cwa_grid_dims": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(_I32)]),
    "cwa_make_reference_cube": (C.c_int, [C.POINTER(SceneDesc), _P, _I32]),
    "cwa_make_dam_break": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(_I32), C.c_float, C.c_float,
                                     C.c_uint64, _P, _I32]),
    "cwa_make_bumps": (C.c_int, [C.POINTER(SceneDesc), _I32, C.c_uint64, _P, _I32, _I32]),
    "cwa_create": (C.c_int, [C.POINTER(SimOptions), C.POINTER(SceneDesc), _I32, C.POINTER(_P)]),
    "cwa_destroy": (C.c_int, [_P]),
    "cwa_upload_particles": (C.c_int, [_P, _I32, _P, _I32]),
    "cwa_download_particles": (C.c_int, [_P, _I32, _P, _I32]),
    "cwa_upload_wave": (C.c_int, [_P, _I32, _P, _P, _I32, _I32]),
    "cwa_download_wave": (C.c_int, [_P, _I32, _P, _P, _I32, _I32]),
    "cwa_wave_reinit": (C.c_int, [_P, _I32]),
    "cwa_step": (C.c_int, [_P, _I32]),
    "cwa_pass_grid": (C.c_int, [_P]),
    "cwa_pass_rho_pres": (C.c_int, [_P]),
    "cwa_pass_force": (C.c_int, [_P]),
    "cwa_pass_integrate": (C.c_int, [_P]),
    "cwa_pass_wave": (C.c_int, [_P]),
    "cwa_wave_advance": (C.c_int, [_P, _I32]),
    "cwa_wave_init_from_image": (C.c_int, [_P, _I32, C.c_void_p, _I32, _I32]),
    "cwa_render_defaults": (C.c_int, [_I32, _I32, C.POINTER(Camera), C.POINTER(RenderParams)]),
    "cwa_render_set_skybox": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa_render": (C.c_int, [_P, _I32, C.POINTER(Camera), C.POINTER(RenderParams), C.c_void_p]),
    "cwa2d_defaults": (C.c_int, [C.POINTER(Params2D)]),
    "cwa2d_create": (C.c_int, [C.POINTER(Params2D), _I32, C.POINTER(_P)]),
    "cwa2d_destroy": (C.c_int, [_P]),
    "cwa2d_reinit": (C.c_int, [_P]),
    "cwa2d_splash": (C.c_int, [_P]),
    "cwa2d_step": (C.c_int, [_P, _I32]),
    "cwa2d_pass": (C.c_int, [_P, _I32]),
    "cwa2d_upload_particles": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa2d_download_particles": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa2d_upload_wave": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa2d_download_wave": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa2d_upload_wave_prev": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa2d_download_wave_prev": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa2d_synchronize": (C.c_int, [_P]),
    "cwa_pbd_defaults": (C.c_int, [C.POINTER(PbdParams)]),
    "cwa_pbd_make_boxes": (C.c_int, [C.POINTER(PbdParams), C.c_uint64, C.c_void_p, _I32]),
    "cwa_pbd_create": (C.c_int, [C.POINTER(PbdParams), _I32, C.POINTER(_P)]),
    "cwa_pbd_destroy": (C.c_int, [_P]),
    "cwa_pbd_upload": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa_pbd_download": (C.c_int, [_P, C.c_void_p, _I32]),
    "cwa_pbd_step": (C.c_int, [_P, _I32]),
    "cwa_pbd_pair_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "cwa_synchronize": (C.c_int, [_P]),
    "cwa_get_step_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "cwa_get_rebuild_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "cwa_get_device_view": (C.c_int, [_P, _I32, C.POINTER(DeviceView)]),
    "cwa_download_grid": (C.c_int, [_P, _I32, _P, _I32, _P, _I32]),
    "cwa_download_deposits": (C.c_int, [_P, _I32, _P, _I32, _I32]),
    "cwa_reduce_totals": (C.c_int, [_P, _I32, _P]),
    "cwa_save": (C.c_int, [_P, C.c_char_p]),
    "cwa_load": (C.c_int, [_P, C.c_char_p]),
    "cwa_set_profiling": (C.c_int, [_P, _I32]),
    "cwa_get_pass_times": (C.c_int, [_P, _P, _I32]),
    "cwa_get_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "cwa_autotune": (C.c_int, [_P, _I32, C.POINTER(TuneReport)]),
    "cwa_autotune_wave": (C.c_int, [_P, _I32, C.POINTER(WaveTuneReport)]),
    "cwa_debug_fail_alloc": (C.c_int, [_I32]),
    "cwa_get_options": (C.c_int, [_P, C.POINTER(SimOptions)]),
    "cwa_scan_workspace_bytes": (C.c_size_t, [_I32]),
    "cwa_exclusive_scan_i32": (C.c_int, [_P, _P, _I32, _P, C.c_size_t, _P]),
    "cwa_exclusive_scan_i32_noalloc": (C.c_int, [_P, _P, _I32, _P]),
    "cwa_scan_status": (C.c_int, [_I32, _P, _P]),
    "cwa_scan_noalloc_status": (C.c_int, [_P]),
    "cwa_grid_status": (C.c_int, [_I32, _I32, _P, _P]),
    "cwa_grid_workspace_bytes": (C.c_size_t, [_I32, _I32]),
    "cwa_grid_build": (C.c_int, [_P, _I32, C.POINTER(C.c_float), C.c_float, C.POINTER(_I32), _P, _P,
                                 _P, _P, C.c_size_t, _P]),
}

_lib = None


class CwaError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {status_str(status)} ({status}) {detail}".rstrip())


def load() -> C.CDLL:
    """Load libcwa.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it first "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def status_str(status: int) -> str:
    return load().cwa_status_str(status).decode()


def last_error() -> str:
    return load().cwa_last_error().decode()


def check(status: int, where: str) -> None:
    if status != CWA_OK:
        raise CwaError(status, where, last_error())


def ptr(a) -> C.c_void_p:
    """Host (numpy) or device (torch) buffer address as a void pointer."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


def declared_functions(header: Path | None = None) -> list[str]:
    """Names of the functions include/cwa.h declares."""
    import re
    header = header or (Path(__file__).resolve().parent.parent / "include" / "cwa.h")
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cwa(?:2d)?_[a-z0-9_]+)\s*\(", text)))
