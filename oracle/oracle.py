"""ctypes binding of the CPU oracle (oracle/cwa_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs.  The product never imports it.
Particles cross this boundary as (n, 16) float64 arrays (pos, vel, force,
extras) for the FP64 passes and as the 64-byte record for the float32 ones.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcwa_oracle.so"

_P = C.c_void_p
_I = C.c_int32
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        protos = {
            "orc_num_threads": (C.c_int, []),
            "orc_set_num_threads": (None, [C.c_int]),
            "orc_exclusive_scan_i32": (None, [_P, _P, _I]),
            "orc_cell_id_f32": (_I, [_P, _P, _P, _P]),
            "orc_grid_build_f32": (None, [_P, _I, _P, _P, _P, _P, _P, _P]),
            "orc_grid_dims": (None, [_P, _P]),
            "orc_scene_defaults": (None, [_I, C.c_float, _P]),
            "orc_scene_set_wave_grid": (None, [_P, _I, _I]),
            "orc_make_reference_cube": (None, [_P, _P, _I]),
            "orc_make_dam_break": (None, [_P, _P, C.c_float, C.c_float, C.c_uint64, _P, _I]),
            "orc_make_bumps": (None, [_P, _I, C.c_uint64, _P, _I, _I]),
            "orc_rho_pres": (None, [_P, _I, _P, _P, _I]),
            "orc_force": (None, [_P, _I, _P, _P, _I]),
            "orc_integrate": (None, [_P, _I, _P, _P, _P]),
            "orc_wave": (None, [_P, _P, _P, _P, _P]),
            "orc_step": (None, [_P, _I, _P, _P, _P, _I, _I]),
            "orc_totals": (None, [_P, _I, _P, _P, _P, _P]),
            "orc_integrate_f32": (None, [_P, _I, _P, _P, _P]),
            "orc_wave_f32": (None, [_P, _P, _P, _P, _P]),
            "orc_wave_init_f32": (None, [_P, _P]),
            "orc_wave_from_image_f32": (None, [C.c_int32, C.c_int32, _P, C.c_int32, C.c_int32, _P]),
            "orc_sample_f32": (C.c_float, [_P, _I, _I, C.c_float, C.c_float]),
            "orc_render": (None, [_P, _I, _P, _I, _I, _P, _P, _P, _I, _P]),
            "orc_shade_particle": (None, [_P, _P, _P, _P, _I, _P, _I, _I, _I, _I, C.c_float, _P, _P]),
            "orc_shade_wave": (None, [_P, _P, _I, _P, C.c_float, _P]),
            "orc2d_init_particles": (None, [_P, _P]),
            "orc2d_wave_init_f32": (None, [_P, _P, _P, _I]),
            "orc2d_wave_iter_f32": (None, [_P, _P, _P, _I]),
            "orc2d_wave1d_init_f32": (None, [_P, _P, _P, _P, _I]),
            "orc2d_wave1d_iter_f32": (None, [_P, _P, _P, _P]),
            "orc2d_density": (None, [_P, _P, _P, _P]),
            "orc2d_force": (None, [_P, _P, _P, _P, _P]),
            "orc_pbd_step": (None, [_P, _P, _I, _I]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _d(desc):
    return C.cast(C.byref(desc), C.c_void_p)


def threads() -> int:
    return load().orc_num_threads()


def set_threads(n: int) -> None:
    load().orc_set_num_threads(n)


# ---------------------------------------------------------------- helpers --
def to_f64(particles: np.ndarray) -> np.ndarray:
    """64-byte particle records -> (n, 16) float64."""
    return np.ascontiguousarray(particles.view(np.float32).reshape(-1, 16), dtype=np.float64)


def to_f32_records(p16: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(p16, dtype=np.float32).reshape(-1, 16)


# ------------------------------------------------------------ integer parts --
def exclusive_scan(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.int32)
    out = np.zeros_like(x)
    load().orc_exclusive_scan_i32(_p(x), _p(out), len(x))
    return out


def cell_edges(desc) -> tuple[float, float, float]:
    z = desc.cell_size_z if desc.cell_size_z > 0 else desc.cell_size
    return (desc.cell_size, desc.cell_size, z)


def grid_dims(desc) -> tuple[int, int, int]:
    dims = np.zeros(3, np.int32)
    load().orc_grid_dims(_d(desc), _p(dims))
    return tuple(int(v) for v in dims)


def grid_build(pos4: np.ndarray, lo, cell, dims):
    """cell: one edge for all axes, or (x, y, z) edges."""
    pos4 = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    lo = np.ascontiguousarray(lo, np.float32)
    cell = np.ascontiguousarray(np.broadcast_to(np.asarray(cell, np.float32), (3,)), np.float32)
    dims = np.ascontiguousarray(dims, np.int32)
    n = len(pos4)
    nc = int(np.prod(dims))
    start = np.zeros(nc + 1, np.int32)
    order = np.zeros(n, np.int32)
    cell_of = np.zeros(n, np.int32)
    load().orc_grid_build_f32(_p(pos4), n, _p(lo), _p(cell), _p(dims), _p(start), _p(order), _p(cell_of))
    return start, order, cell_of


# ---------------------------------------------------------------- scenes --
def scene_defaults(preset: int, spacing: float, desc_type):
    d = desc_type()
    load().orc_scene_defaults(preset, spacing, _d(d))
    return d


def scene_set_wave_grid(desc, nx: int, nz: int) -> None:
    load().orc_scene_set_wave_grid(_d(desc), nx, nz)


def make_reference_cube(desc, n: int) -> np.ndarray:
    out = np.zeros((n, 16), np.float32)
    load().orc_make_reference_cube(_d(desc), _p(out), n)
    return out


def make_dam_break(desc, dims, spacing, jitter, seed, n) -> np.ndarray:
    out = np.zeros((n, 16), np.float32)
    d = np.ascontiguousarray(dims, np.int32)
    load().orc_make_dam_break(_d(desc), _p(d), spacing, jitter, seed, _p(out), n)
    return out


def make_bumps(desc, n_bumps, seed, nx, nz) -> np.ndarray:
    out = np.zeros((nz, nx), np.float32)
    load().orc_make_bumps(_d(desc), n_bumps, seed, _p(out), nx, nz)
    return out


# ------------------------------------------------------------ FP64 passes --
def rho_pres(desc, p16: np.ndarray, u_n: np.ndarray, brute=False) -> None:
    load().orc_rho_pres(_d(desc), len(p16), _p(p16), _p(np.ascontiguousarray(u_n, np.float64)), int(brute))


def force(desc, p16: np.ndarray, u_n: np.ndarray, brute=False) -> None:
    load().orc_force(_d(desc), len(p16), _p(p16), _p(np.ascontiguousarray(u_n, np.float64)), int(brute))


def integrate(desc, p16: np.ndarray, u_n: np.ndarray, deposits: np.ndarray | None = None) -> None:
    load().orc_integrate(_d(desc), len(p16), _p(p16), _p(np.ascontiguousarray(u_n, np.float64)),
                         _p(deposits))


def wave(desc, u_n, u_nm1, deposits=None) -> np.ndarray:
    a = np.ascontiguousarray(u_n, np.float64)
    b = np.ascontiguousarray(u_nm1, np.float64)
    out = np.zeros_like(a)
    load().orc_wave(_d(desc), _p(a), _p(b), _p(out), _p(deposits))
    return out


def step(desc, p16: np.ndarray, u_n: np.ndarray, u_nm1: np.ndarray, n_steps: int, brute=False) -> None:
    """In place: p16 (n,16) f64, u_n / u_nm1 f64 (rotated each step)."""
    for a in (p16, u_n, u_nm1):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    load().orc_step(_d(desc), len(p16), _p(p16), _p(u_n), _p(u_nm1), n_steps, int(brute))


def totals(desc, p16, u_n, u_nm1) -> np.ndarray:
    out = np.zeros(8, np.float64)
    load().orc_totals(_d(desc), len(p16), _p(p16), _p(np.ascontiguousarray(u_n, np.float64)),
                      _p(np.ascontiguousarray(u_nm1, np.float64)), _p(out))
    return out


# ------------------------------------------------------- FP32-exact passes --
def integrate_f32(desc, p16f: np.ndarray, u_n: np.ndarray, with_deposits=True):
    p16f = np.ascontiguousarray(p16f, np.float32).copy()
    dep = np.zeros((desc.wave_nz, desc.wave_nx), np.int64) if with_deposits else None
    load().orc_integrate_f32(_d(desc), len(p16f), _p(p16f), _p(np.ascontiguousarray(u_n, np.float32)),
                             _p(dep))
    return p16f, dep


def wave_f32(desc, u_n, u_nm1, deposits=None) -> np.ndarray:
    a = np.ascontiguousarray(u_n, np.float32)
    b = np.ascontiguousarray(u_nm1, np.float32)
    out = np.zeros_like(a)
    dep = None if deposits is None else np.ascontiguousarray(deposits, np.int64)
    load().orc_wave_f32(_d(desc), _p(a), _p(b), _p(out), _p(dep))
    return out


def wave_from_image_f32(nx: int, nz: int, rgba: np.ndarray) -> np.ndarray:
    """InitFromImage on an (h, w, 4) uint8 texture (row 0 = texture row 0)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    out = np.zeros((nz, nx), np.float32)
    load().orc_wave_from_image_f32(nx, nz, _p(img), w, h, _p(out))
    return out


def wave_init_f32(desc) -> np.ndarray:
    out = np.zeros((desc.wave_nz, desc.wave_nx), np.float32)
    load().orc_wave_init_f32(_d(desc), _p(out))
    return out


def sample_f32(u, s, t) -> float:
    u = np.ascontiguousarray(u, np.float32)
    return float(load().orc_sample_f32(_p(u), u.shape[1], u.shape[0], s, t))


def omp_threads_env() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", "0") or 0)


def render(pos4: np.ndarray, wave: np.ndarray, camera, params, sky: np.ndarray | None = None) -> np.ndarray:
    """One frame (height, width, 4) uint8, row 0 at the bottom.  pos4: (n, 4)
    float32 positions in upload order; wave: (nz, nx) u^n; camera / params:
    the ABI's cwa_camera / cwa_render_params ctypes structures; sky: (6, S, S, 4)."""
    p = np.ascontiguousarray(pos4, np.float32)
    u = np.ascontiguousarray(wave, np.float32)
    out = np.zeros((params.height, params.width, 4), np.uint8)
    sk = None if sky is None else np.ascontiguousarray(sky, np.uint8)
    load().orc_render(_p(p), p.shape[0], _p(u), u.shape[1], u.shape[0], C.cast(C.pointer(camera), C.c_void_p),
                      C.cast(C.pointer(params), C.c_void_p), _p(sk), 0 if sk is None else sk.shape[1], _p(out))
    return out


def shade_particle(inv_p, inv_v, eye, sky, sky_size, depth, px: int, py: int, r: float, pp) -> np.ndarray:
    """particle_fs.glsl pass 0 for one fragment (rgba before blending)."""
    f = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    out = np.zeros(4, np.float32)
    d = f(depth)
    skyb = None if sky is None else np.ascontiguousarray(sky, np.uint8)
    load().orc_shade_particle(_p(f(inv_p)), _p(f(inv_v)), _p(f(eye)), _p(skyb), sky_size, _p(d), d.shape[1],
                              d.shape[0], px, py, r, _p(f(pp)), _p(out))
    return out


def shade_wave(eye, sky, sky_size, p, v: float) -> np.ndarray:
    """wave_fs.glsl for one fragment (rgba before blending)."""
    f = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    out = np.zeros(4, np.float32)
    skyb = None if sky is None else np.ascontiguousarray(sky, np.uint8)
    load().orc_shade_wave(_p(f(eye)), _p(skyb), sky_size, _p(f(p)), v, _p(out))
    return out


# ---- the 2D solver family ----
def _pp(params):
    return C.cast(C.pointer(params), C.c_void_p)


def init_particles_2d(params, dtype) -> np.ndarray:
    out = np.zeros(params.n_particles, dtype)
    load().orc2d_init_particles(_pp(params), _p(out))
    return out


def wave_init_2d_f32(params, prev=None, splash=False) -> np.ndarray:
    inp = np.zeros((params.wave_cells, 4), np.float32) if prev is None else np.ascontiguousarray(prev, np.float32)
    out = np.zeros((params.wave_cells, 4), np.float32)
    load().orc2d_wave_init_f32(_pp(params), _p(inp), _p(out), int(splash))
    return out


def wave_iter_2d_f32(params, cells4, phase: int, out_prev=None) -> np.ndarray:
    """One Lax-Wendroff phase; out_prev = the write buffer's previous contents."""
    inp = np.ascontiguousarray(cells4, np.float32)
    out = np.zeros_like(inp) if out_prev is None else np.ascontiguousarray(out_prev, np.float32).copy()
    load().orc2d_wave_iter_f32(_pp(params), _p(inp), _p(out), phase)
    return out


def wave1d_init_2d_f32(params, mode: int, cur=None, prev=None) -> np.ndarray:
    """Wave1D MODE_INIT_0 / MODE_INIT_1 on (newest, older) fields."""
    n = params.wave_cells
    c = np.zeros((n, 4), np.float32) if cur is None else np.ascontiguousarray(cur, np.float32)
    q = np.zeros((n, 4), np.float32) if prev is None else np.ascontiguousarray(prev, np.float32)
    out = np.zeros((n, 4), np.float32)
    load().orc2d_wave1d_init_f32(_pp(params), _p(c), _p(q), _p(out), int(mode))
    return out


def wave1d_iter_2d_f32(params, cur, prev) -> np.ndarray:
    """One Wave1D MODE_ITERATE step with free boundaries."""
    c = np.ascontiguousarray(cur, np.float32)
    q = np.ascontiguousarray(prev, np.float32)
    out = np.zeros_like(c)
    load().orc2d_wave1d_iter_f32(_pp(params), _p(c), _p(q), _p(out))
    return out


def density_2d(params, particles, wave4) -> np.ndarray:
    inp = np.ascontiguousarray(particles)
    out = np.zeros_like(inp)
    load().orc2d_density(_pp(params), _p(inp), _p(np.ascontiguousarray(wave4, np.float32)), _p(out))
    return out


def force_2d(params, particles, wave4, grid_from=None) -> np.ndarray:
    """ComputeForces on `particles` over the grid of `grid_from` (the
    substep's state before the density pass; default: `particles`)."""
    inp = np.ascontiguousarray(particles)
    src = None if grid_from is None else np.ascontiguousarray(grid_from)
    out = np.zeros_like(inp)
    load().orc2d_force(_pp(params), _p(inp), _p(src), _p(np.ascontiguousarray(wave4, np.float32)), _p(out))
    return out


def pbd_step(params, boxes, steps: int):
    """`steps` PBD frames of a copy of `boxes` (numpy records, 128 bytes each)."""
    out = np.ascontiguousarray(boxes).copy()
    load().orc_pbd_step(_pp(params), _p(out), len(out), steps)
    return out
