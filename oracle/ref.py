"""The reference's compute shaders run on the CPU: ctypes access to
oracle/_ref/libcwa_ref_shaders.so, plus the seeded inputs the golden
fixtures of tests/golden/ref_shader_outputs.npz are computed on.

TEST INFRASTRUCTURE ONLY.  The library is compiled from the reference
checkout's own shader source (CoupledWaterAnimation/rho_pres_comp.glsl,
force_comp.glsl, integrate_comp.glsl, wave_comp.glsl) by
oracle/ref_shaders/Makefile; it exists only where that checkout does.  The
fixtures it produced are committed, so the checks that use them run
anywhere.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libcwa_ref_shaders.so"
# the reference checkout of this container (absent elsewhere); CWA_REFERENCE overrides it
DEFAULT_REFERENCE = Path("/root/reference")

NUM_PARTICLES = 20480  # the shaders' NUM_PARTICLES (rho_pres_comp.glsl:4)
F32, F64 = 0, 1


class Uniforms(C.Structure):
    """ref_uniforms (oracle/ref_shaders/ref_shaders.h): the uniform blocks of
    Main.cpp:184-204 as the shaders declare them."""
    _fields_ = [("mass", C.c_float), ("smoothing_coeff", C.c_float), ("visc", C.c_float),
                ("resting_rho", C.c_float), ("upper", C.c_float * 4), ("lower", C.c_float * 4),
                ("attributes", C.c_float * 4), ("mesh_ws_pos", C.c_float * 4), ("time", C.c_float),
                ("mode", C.c_int32)]


class Uniforms2D(C.Structure):
    """ref2d_uniforms (oracle/ref_shaders/ref_shaders.h)."""
    _fields_ = [("time", C.c_float), ("bottom", C.c_float), ("grid_cells", C.c_int32 * 2),
                ("extent_max", C.c_float * 2), ("wave_lambda", C.c_float), ("dx", C.c_float),
                ("atten", C.c_float), ("beta", C.c_float), ("boundary", C.c_float * 2)]


def uniforms_2d(params) -> Uniforms2D:
    """The 2D family's uniforms from a cwa2d_params (its defaults are the
    reference app's values)."""
    u = Uniforms2D()
    u.time = 0.0
    u.bottom = params.bottom
    u.grid_cells[:] = list(params.grid_cells)
    u.extent_max[:] = list(params.view_size)
    u.wave_lambda = params.wave_lambda
    u.dx = params.wave_dx
    u.atten = params.wave_atten
    u.beta = params.wave_beta
    return u


class PbdParams(C.Structure):
    """ref_pbd_params (oracle/ref_shaders/ref_shaders.h)."""
    _fields_ = [("grid_cells", C.c_int32 * 3), ("lo", C.c_float * 3), ("hi", C.c_float * 3), ("g", C.c_float * 3),
                ("dt", C.c_float), ("damping", C.c_float), ("k", C.c_float), ("k_static", C.c_float),
                ("sleep_thresh", C.c_float), ("mu_k", C.c_float), ("mu_s", C.c_float), ("e", C.c_float),
                ("substeps", C.c_int32)]


def pbd_params(params) -> PbdParams:
    """The shader's Params block and grid from a cwa_pbd_params."""
    q = PbdParams()
    q.grid_cells[:] = list(params.grid_cells)
    q.lo[:] = list(params.extents_lo)
    q.hi[:] = list(params.extents_hi)
    q.g[:] = list(params.g)
    for f in ("dt", "damping", "k", "k_static", "sleep_thresh", "mu_k", "mu_s", "e", "substeps"):
        setattr(q, f, getattr(params, f))
    return q


def pbd(prec: int, boxes32: np.ndarray, frames: int, q: PbdParams) -> np.ndarray:
    """`frames` frames of the PBD shader on (n, 32) box records."""
    a = np.ascontiguousarray(boxes32, np.float64).copy()
    if load().ref_pbd(prec, _dp(a), len(a), frames, C.byref(q)) != 0:
        raise ValueError("ref_pbd needs nx == nz and a power-of-two cell count")
    return a


class RenderInputs(C.Structure):
    """ref_render_inputs (oracle/ref_shaders/ref_shaders.h)."""
    _fields_ = [("P", C.c_float * 16), ("V", C.c_float * 16), ("PV", C.c_float * 16), ("eye", C.c_float * 3),
                ("sky", C.c_void_p), ("sky_size", C.c_int32), ("depth_image", C.c_void_p), ("w", C.c_int32),
                ("h", C.c_int32)]


def particle_fragment(inp: RenderInputs, pp, depth: float, px: float, py: float, point_coord):
    """particle_fs.glsl pass 0 for one fragment: (rgba, discarded)."""
    out = np.zeros(4, np.float32)
    a = np.ascontiguousarray(pp, np.float32)
    pc = np.ascontiguousarray(point_coord, np.float32)
    d = load().ref_particle_fragment(C.byref(inp), _fp(a), depth, px, py, _fp(pc), _fp(out))
    return out, bool(d)


def wave_fragment(inp: RenderInputs, pw, nw, v: float) -> np.ndarray:
    """wave_fs.glsl for one fragment."""
    out = np.zeros(4, np.float32)
    load().ref_wave_fragment(C.byref(inp), _fp(np.ascontiguousarray(pw, np.float32)),
                             _fp(np.ascontiguousarray(nw, np.float32)), v, _fp(out))
    return out


def reference_root() -> Path | None:
    ref = Path(os.environ.get("CWA_REFERENCE", str(DEFAULT_REFERENCE)))
    return ref if (ref / "CoupledWaterAnimation" / "rho_pres_comp.glsl").is_file() else None


def build(verbose: bool = False) -> Path | None:
    """Compile the shaders when the reference checkout is present; returns
    the library path, or None without a checkout."""
    ref = reference_root()
    if ref is None:
        return None
    subprocess.run(["make", "-s" if not verbose else "-w", "-C", str(HERE / "ref_shaders"), f"REF={ref}"],
                   check=True)
    return LIB_PATH


_lib = None


def load():
    """The compiled shaders, or None where they were not built."""
    global _lib
    if _lib is None and LIB_PATH.is_file():
        lib = C.CDLL(str(LIB_PATH))
        dp, fp = C.POINTER(C.c_double), C.POINTER(C.c_float)
        for name in ("ref_rho_pres", "ref_force", "ref_integrate"):
            f = getattr(lib, name)
            f.argtypes = [C.c_int32, dp, C.c_int32, fp, C.c_int32, C.c_int32, C.POINTER(Uniforms)]
            f.restype = C.c_int32
        lib.ref_wave.argtypes = [C.c_int32, dp, dp, dp, C.c_int32, C.c_int32, fp, C.c_int32, C.c_int32,
                                 C.POINTER(Uniforms)]
        lib.ref_wave.restype = C.c_int32
        ip = C.POINTER(C.c_int32)
        lib.ref_exclusive_scan.argtypes = [ip, ip, C.c_int32]
        lib.ref_exclusive_scan.restype = C.c_int32
        lib.ref_grid_build.argtypes = [fp, C.c_int32, fp, fp, fp, ip, ip, ip, ip]
        lib.ref_grid_build.restype = C.c_int32
        u2 = C.POINTER(Uniforms2D)
        lib.ref2d_sph.argtypes = [C.c_int32, C.c_int32, dp, dp, C.c_int32, fp, C.c_int32, u2]
        lib.ref2d_sph.restype = C.c_int32
        lib.ref2d_substep.argtypes = [C.c_int32, dp, dp, dp, C.c_int32, fp, C.c_int32, u2]
        lib.ref2d_substep.restype = C.c_int32
        lib.ref2d_field.argtypes = [C.c_int32, C.c_int32, fp, fp, fp, C.c_int32, fp, C.c_int32, u2]
        lib.ref2d_field.restype = C.c_int32
        lib.ref_pbd.argtypes = [C.c_int32, dp, C.c_int32, C.c_int32, C.POINTER(PbdParams)]
        lib.ref_pbd.restype = C.c_int32
        ri = C.POINTER(RenderInputs)
        lib.ref_particle_fragment.argtypes = [ri, fp, C.c_float, C.c_float, C.c_float, fp, fp]
        lib.ref_particle_fragment.restype = C.c_int32
        lib.ref_wave_fragment.argtypes = [ri, fp, fp, C.c_float, fp]
        lib.ref_wave_fragment.restype = C.c_int32
        _lib = lib
    return _lib


def uniforms(desc, mode: int = 0) -> Uniforms:
    """The uniforms of a REFERENCE_3D scene description, with Main.cpp's
    values for the fields the description does not carry (upper.w = 500,
    lower.w = 50, Main.cpp:194-195)."""
    u = Uniforms()
    u.mass = desc.mass
    u.smoothing_coeff = np.float32(desc.smoothing_length) / np.float32(desc.particle_radius)
    u.visc = desc.visc
    u.resting_rho = desc.rest_rho
    u.upper[:] = [desc.box_hi[0], desc.box_hi[1], desc.box_hi[2], 500.0]
    u.lower[:] = [desc.box_lo[0], desc.box_lo[1], desc.box_lo[2], 50.0]
    u.attributes[:] = [desc.wave_lambda, desc.wave_atten, desc.wave_beta, desc.wave_mode]
    u.time = 0.0
    u.mode = mode
    return u


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fp(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _particle_pass(name: str, prec: int, p16: np.ndarray, wave: np.ndarray, u: Uniforms) -> np.ndarray:
    lib = load()
    out = np.ascontiguousarray(p16, dtype=np.float64).copy()
    w = np.ascontiguousarray(wave, dtype=np.float32)
    rc = getattr(lib, name)(prec, _dp(out), len(out), _fp(w), w.shape[1], w.shape[0], C.byref(u))
    if rc != 0:
        raise ValueError(f"{name}: {len(out)} particles (the shader loops over {NUM_PARTICLES})")
    return out


def rho_pres(prec, p16, wave, u):
    return _particle_pass("ref_rho_pres", prec, p16, wave, u)


def force(prec, p16, wave, u):
    return _particle_pass("ref_force", prec, p16, wave, u)


def integrate(prec, p16, wave, u):
    return _particle_pass("ref_integrate", prec, p16, wave, u)


def wave(prec, u_n, u_nm1, uni: Uniforms, init_rgba: np.ndarray | None = None) -> np.ndarray:
    lib = load()
    a = np.ascontiguousarray(u_n, dtype=np.float64)
    b = np.ascontiguousarray(u_nm1, dtype=np.float64)
    out = np.zeros_like(a)
    img = None if init_rgba is None else np.ascontiguousarray(init_rgba, dtype=np.float32)
    iw, ih = (0, 0) if img is None else (img.shape[1], img.shape[0])
    rc = lib.ref_wave(prec, _dp(a), _dp(b), _dp(out), a.shape[1], a.shape[0], _fp(img), iw, ih, C.byref(uni))
    if rc != 0:
        raise ValueError("ref_wave failed")
    return out


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def exclusive_scan(x: np.ndarray) -> np.ndarray:
    """ParallelScan::Compute with prefix_sum_cs.glsl (n a power of two)."""
    a = np.ascontiguousarray(x, np.int32)
    out = np.zeros_like(a)
    if load().ref_exclusive_scan(_ip(a), _ip(out), len(a)) != 0:
        raise ValueError("the reference scan needs a power-of-two length")
    return out


def grid_build(pos4: np.ndarray, lo, hi, cell, dims):
    """ugrid_particles_cs.glsl COMPUTE_COUNTS, the scan, INSERT_PARTICLES:
    (counts, offsets, index list).  dims: (nx, ny, nz) with nx == nz and a
    power-of-two product (what the reference's Index() and scan support)."""
    p = np.ascontiguousarray(pos4, np.float32)
    f = lambda v: np.ascontiguousarray(v, np.float32)  # noqa: E731
    d = np.ascontiguousarray(dims, np.int32)
    nc = int(np.prod(d))
    counts, offsets, lst = np.zeros(nc, np.int32), np.zeros(nc, np.int32), np.zeros(len(p), np.int32)
    lo_, hi_, cell_ = f(lo), f(hi), f(cell)
    rc = load().ref_grid_build(_fp(p), len(p), _fp(lo_), _fp(hi_), _fp(cell_), _ip(d), _ip(counts), _ip(offsets),
                               _ip(lst))
    if rc != 0:
        raise ValueError("the reference grid needs nx == nz and a power-of-two cell count")
    return counts, offsets, lst


def sph2d(prec: int, mode: int, p12: np.ndarray, wave4: np.ndarray, u: Uniforms2D) -> np.ndarray:
    """The grid of p12, then one SphWaveKoschier2D mode over it."""
    a = np.ascontiguousarray(p12, np.float64)
    out = np.zeros_like(a)
    w = np.ascontiguousarray(wave4, np.float32)
    if load().ref2d_sph(prec, mode, _dp(a), _dp(out), len(a), _fp(w), len(w), C.byref(u)) != 0:
        raise ValueError("ref2d_sph failed")
    return out


def substep2d(prec: int, p12: np.ndarray, wave4: np.ndarray, u: Uniforms2D):
    """One SphUgrid::Compute substep: (after density, after forces)."""
    a = np.ascontiguousarray(p12, np.float64)
    dens, force = np.zeros_like(a), np.zeros_like(a)
    w = np.ascontiguousarray(wave4, np.float32)
    if load().ref2d_substep(prec, _dp(a), _dp(dens), _dp(force), len(a), _fp(w), len(w), C.byref(u)) != 0:
        raise ValueError("ref2d_substep failed")
    return dens, force


def field2d(kind: int, mode: int, in0, in1, out_prev, u: Uniforms2D, init4=None) -> np.ndarray:
    """One Shallow1D (kind 0) or Wave1D (kind 1) dispatch; out_prev: the
    output image's contents before it."""
    a = np.ascontiguousarray(in0, np.float32)
    b = np.ascontiguousarray(a if in1 is None else in1, np.float32)
    out = np.ascontiguousarray(out_prev, np.float32).copy()
    img = None if init4 is None else np.ascontiguousarray(init4, np.float32)
    load().ref2d_field(kind, mode, _fp(a), _fp(b), _fp(out), len(a), _fp(img), 0 if img is None else len(img),
                       C.byref(u))
    return out


# ----------------------------------------------------------- seeded inputs ----
def uniform01(seed: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from splitmix64 of (seed, index): integer
    arithmetic only, so every host makes the same numbers."""
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (i + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _u32(seed: int, n: int, lo: float, hi: float) -> np.ndarray:
    return (lo + (hi - lo) * uniform01(seed, n)).astype(np.float32)


def sph_state() -> np.ndarray:
    """20480 particle records (float32 values): the reference's 64 x 5 x 64
    cube (Main.cpp:735-778, spacing 2 * 0.85 * 0.005) with each position
    jittered by up to 0.3 spacings, velocities in [-0.3, 0.3), a previous
    step's force in [-500, 500) and the initial extras (1000, 0, 500, 50)."""
    n = NUM_PARTICLES
    sp = np.float32(2.0) * np.float32(0.85) * np.float32(0.005)
    ii, jj, kk = np.meshgrid(np.arange(64), np.arange(5), np.arange(64), indexing="ij")
    p = np.zeros((n, 16), np.float32)
    p[:, 0] = ii.reshape(-1).astype(np.float32) * sp
    p[:, 1] = jj.reshape(-1).astype(np.float32) * sp
    p[:, 2] = kk.reshape(-1).astype(np.float32) * sp
    for c in range(3):
        p[:, c] += _u32(101 + c, n, -0.3, 0.3) * sp
        p[:, 4 + c] = _u32(201 + c, n, -0.3, 0.3)
        p[:, 8 + c] = _u32(301 + c, n, -500.0, 500.0)
    p[:, 3] = 1.0
    p[:, 11] = _u32(304, n, -10.0, 10.0)
    p[:, 12:16] = [1000.0, 0.0, 500.0, 50.0]
    return p


def integrate_state(n: int = 1024) -> np.ndarray:
    """n particle records spread over the reference box and a margin past its
    walls (x, z in [-0.02, 0.5), y in [-0.04, 1.06)), velocities in [-5, 5)
    with every 17th scaled past the foam speed 25, forces in [-3e4, 3e4),
    rho in [900, 1100), p in [0, 4e5)."""
    p = np.zeros((n, 16), np.float32)
    p[:, 0] = _u32(401, n, -0.02, 0.5)
    p[:, 1] = _u32(402, n, -0.04, 1.06)
    p[:, 2] = _u32(403, n, -0.02, 0.5)
    p[:, 3] = 1.0
    for c in range(3):
        p[:, 4 + c] = _u32(411 + c, n, -5.0, 5.0)
        p[:, 8 + c] = _u32(421 + c, n, -3e4, 3e4)
    p[::17, 4:7] *= np.float32(8.0)
    p[:, 11] = _u32(424, n, -10.0, 10.0)
    p[:, 12] = _u32(431, n, 900.0, 1100.0)
    p[:, 13] = _u32(432, n, 0.0, 4e5)
    p[:, 14:16] = [500.0, 50.0]
    return p


def height_field(seed: int, w: int, h: int, amp: float = 0.02) -> np.ndarray:
    """A w x h field: two Gaussian bumps of height amp plus noise of amp/4."""
    x = (np.arange(w, dtype=np.float64) + 0.5) / w
    z = (np.arange(h, dtype=np.float64) + 0.5) / h
    X, Z = np.meshgrid(x, z)
    f = amp * (np.exp(-((X - 0.3) ** 2 + (Z - 0.4) ** 2) / 0.02) + 0.6 * np.exp(-((X - 0.75) ** 2 + (Z - 0.7) ** 2) / 0.01))
    f += (amp / 4) * (uniform01(seed, w * h).reshape(h, w) - 0.5)
    return f.astype(np.float32)


def grid_points(seed: int, n: int, hi) -> np.ndarray:
    """n float4 points over [-0.05, hi + 0.05) per axis (some outside the grid,
    to be clamped), every 101st on a cell face (z = 0.25), w = 1."""
    p = np.ones((n, 4), np.float32)
    for c in range(3):
        p[:, c] = _u32(seed + c, n, -0.05, float(hi[c]) + 0.05)
    p[::101, 2] = np.float32(0.25)
    return p


def lattice_points(seed: int, dims, spacing: float, jitter: float) -> np.ndarray:
    """A jittered lattice of float4 points (a dam-break block), w = 1."""
    ii, jj, kk = np.meshgrid(*(np.arange(d) for d in dims), indexing="ij")
    n = ii.size
    p = np.ones((n, 4), np.float32)
    for c, g in enumerate((ii, jj, kk)):
        p[:, c] = (np.float32(spacing) * (g.reshape(-1).astype(np.float32) + np.float32(0.5))
                   + _u32(seed + c, n, -jitter, jitter) * np.float32(spacing))
    return p


# grid cases of the fixtures: points, lo, hi, cubic cell edge, dims (nx == nz, 2^k cells)
GRID_CASES = {
    "grid_a": (lambda: grid_points(501, 20000, (1.0, 0.5, 1.0)), (0.0, 0.0, 0.0), (1.0, 0.5, 1.0), 1.0 / 16,
               (16, 8, 16)),
    "grid_b": (lambda: lattice_points(511, (24, 20, 24), 0.02, 0.3), (0.0, 0.0, 0.0), (0.64, 0.64, 0.64), 0.02,
               (32, 32, 32)),
}


def scan_inputs() -> dict[str, np.ndarray]:
    """The scan cases: the reference's ParallelScanTest vector
    (SphWave2D/ParallelScan.cpp:129), counts in [0, 40) of length 2^10, and
    values in [0, 10^4) of length 2^14."""
    return {
        "scan_kat": np.array([1, 0, 1, 0, 1, 2, 1, 2, 1, 2, 0, 1, 0, 2, 1, 0], np.int32),
        "scan_1k": (uniform01(521, 1 << 10) * 40).astype(np.int32),
        "scan_16k": (uniform01(522, 1 << 14) * 10000).astype(np.int32),
    }


def sph2d_state(params) -> np.ndarray:
    """params.n_particles records of 12 float32 (pos, vel, acc): the 2D app's
    initial lattice (InitParticle, SphWaveKoschier2D_grid_cs.glsl:308-333)
    jittered by up to 0.03, velocities in [-1, 1), every 7th particle
    disabled (pos.w = 0), density 1000; then particles 0-7 moved past the
    grid's extents (x <= 0, x >= 9.6, y >= 9.6: in no cell list) and
    particles 8-15 below the floor plane (the unpenetrate branch)."""
    n, cols = params.n_particles, params.init_columns
    rows = n // cols
    R = np.float32(params.particle_radius)
    H = np.float32(4.0) * R
    vw, vh = np.float32(params.view_size[0]), np.float32(params.view_size[1])
    ix = np.arange(n)
    p = np.zeros((n, 12), np.float32)
    p[:, 0] = vw * ((ix % cols).astype(np.float32) / np.float32(cols)) + R
    p[:, 1] = (np.float32(18.0) * H) * ((ix // cols).astype(np.float32) / np.float32(rows)) + (
        (np.float32(0.5) * vh - np.float32(15.0) * R) + R)
    p[:, 0] += _u32(601, n, -0.03, 0.03)
    p[:, 1] += _u32(602, n, -0.03, 0.03)
    p[:, 3] = 1.0
    p[::7, 3] = 0.0
    p[:, 4] = _u32(603, n, -1.0, 1.0)
    p[:, 5] = _u32(604, n, -1.0, 1.0)
    p[:, 11] = 1000.0
    p[0:8, 0] = np.array([-0.01, -0.002, 0.0, 9.6, 9.61, 4.0, 5.0, 6.0], np.float32)
    p[5:8, 1] = np.array([9.6, 9.7, 10.0], np.float32)
    p[8:16, 1] = np.float32(0.5) * vh - np.float32(15.0) * R + _u32(605, 8, -0.2, 0.0)
    return p


def shallow_field(params) -> np.ndarray:
    """A shallow-water state (h, uh, h_half, uh_half) for the SPH's wave
    sampling: h = 4.8 plus a bump, uh up to 0.5 h so that |uh / h| crosses
    the 0.05 enable threshold."""
    n = params.wave_cells
    x = (np.arange(n) + 0.5) / n
    f = np.zeros((n, 4), np.float32)
    f[:, 0] = (4.8 + 0.6 * np.exp(-((x - 0.4) ** 2) / 0.01)).astype(np.float32)
    f[:, 1] = (f[:, 0] * (uniform01(611, n) - 0.5)).astype(np.float32)
    return f


def pbd_boxes(params, n: int | None = None) -> np.ndarray:
    """(n, 32) float32 box records (PbdObj) as GridTestPbdGpu3D::Init lays
    them out: positions 0.5 U(-1, 1)^3, velocities 0.1 U(-1, 1)^3, half widths
    U(0.15, 0.45) cell edges per axis, 1 / mass = 1 / (hw.x hw.y hw.z), white."""
    n = params.n_boxes if n is None else n
    b = np.zeros((n, 32), np.float32)
    b[:, 0:4] = 1.0
    edge = [(params.extents_hi[a] - params.extents_lo[a]) / params.grid_cells[a] for a in range(3)]
    for a in range(3):
        b[:, 4 + a] = _u32(701 + a, n, -0.5, 0.5)
        b[:, 8 + a] = _u32(711 + a, n, -0.1, 0.1)
        b[:, 24 + a] = _u32(721 + a, n, 0.15, 0.45) * np.float32(edge[a])
    b[:, 7] = 1.0
    b[:, 28] = np.float32(1.0) / (b[:, 24] * b[:, 25] * b[:, 26])
    return b


def fixture_inputs(splash_rgba8: np.ndarray) -> dict[str, np.ndarray]:
    """Every input of tests/golden/ref_shader_outputs.npz (its cases are
    listed in tests/golden/make_ref_shader_golden.py).  splash_rgba8: the
    reference's splash init texture, (64, 64, 4) uint8."""
    un64 = height_field(11, 64, 64, amp=0.4)
    un67 = height_field(13, 67, 45, amp=0.4)
    return {
        "sph": sph_state(),
        "sph_wave": height_field(7, 64, 64),
        "integ": integrate_state(512),
        "evolve64_un": un64,
        "evolve64_unm1": (un64 * np.float32(0.93)).astype(np.float32),
        "evolve67_un": un67,
        "evolve67_unm1": (un67 * np.float32(0.93)).astype(np.float32),
        # GL's UNORM8 -> float: c / 255, rounded once
        "image_rgba": (np.asarray(splash_rgba8).astype(np.float64) / 255.0).astype(np.float32),
        **{name: case[0]() for name, case in GRID_CASES.items()},
        **scan_inputs(),
        **sph2d_inputs(),
        **pbd_inputs(),
        **render_inputs(),
    }


def _persp(fovy: float, aspect: float, zn: float, zf: float) -> np.ndarray:
    f = 1.0 / np.tan(fovy / 2)
    return np.array([[f / aspect, 0, 0, 0], [0, f, 0, 0], [0, 0, (zf + zn) / (zn - zf), 2 * zf * zn / (zn - zf)],
                     [0, 0, -1, 0]], np.float64)


def _look_at(eye, center, up) -> np.ndarray:
    fwd = center - eye
    fwd = fwd / np.linalg.norm(fwd)
    s = np.cross(fwd, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, fwd)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -fwd
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, fwd @ eye
    return m


def render_inputs(n: int = 2000) -> dict[str, np.ndarray]:
    """Fragment-shader inputs: a camera (P, V and their inverses, float32,
    row-major), an 8^2 cube map of seeded RGBA8 texels, a 64 x 48 pass-2
    depth image, and n fragments of each shader: window pixel, point
    coordinate (about a fifth land outside the sprite and are discarded) and
    particle position for particle_fs; world position and wave sample for
    wave_fs."""
    w, h = 64, 48
    eye = np.array([0.3, 0.8, 1.6])
    P = _persp(0.8, w / h, 0.1, 100.0).astype(np.float32)
    V = _look_at(eye, np.array([0.25, 0.0, 0.25]), np.array([0.0, 1.0, 0.0])).astype(np.float32)
    u = lambda seed, k, lo, hi: _u32(seed, k, lo, hi)  # noqa: E731
    return {
        "rfs_P": P, "rfs_V": V,
        "rfs_PV": (P.astype(np.float64) @ V.astype(np.float64)).astype(np.float32),
        "rfs_inv_p": np.linalg.inv(P.astype(np.float64)).astype(np.float32),
        "rfs_inv_v": np.linalg.inv(V.astype(np.float64)).astype(np.float32),
        "rfs_eye": eye.astype(np.float32),
        "rfs_sky": (uniform01(801, 6 * 8 * 8 * 4) * 256).astype(np.uint8).reshape(6, 8, 8, 4),
        "rfs_depth": u(802, w * h, 0.2, 0.9).reshape(h, w),
        "rfs_px": (uniform01(803, n) * w).astype(np.int32),
        "rfs_py": (uniform01(804, n) * h).astype(np.int32),
        "rfs_pc": np.stack([u(805, n, 0.0, 1.0), u(806, n, 0.0, 1.0)], axis=1),
        "rfs_pp": np.stack([u(807 + c, n, 0.0, 0.5) for c in range(3)], axis=1),
        "rfs_pw": np.stack([u(811 + c, n, -0.5, 1.0) for c in range(3)], axis=1),
        "rfs_v": u(814, n, -0.2, 1.0),
    }


def render_inputs_struct(x: dict[str, np.ndarray]) -> RenderInputs:
    """The RenderInputs of render_inputs() (the arrays must stay alive)."""
    inp = RenderInputs()
    inp.P[:] = x["rfs_P"].T.ravel().tolist()  # GLSL matrices are column-major
    inp.V[:] = x["rfs_V"].T.ravel().tolist()
    inp.PV[:] = x["rfs_PV"].T.ravel().tolist()
    inp.eye[:] = x["rfs_eye"].tolist()
    inp.sky, inp.sky_size = x["rfs_sky"].ctypes.data, x["rfs_sky"].shape[1]
    inp.depth_image = x["rfs_depth"].ctypes.data
    inp.h, inp.w = x["rfs_depth"].shape
    return inp


def point_radius(pc: np.ndarray) -> np.ndarray:
    """length(gl_PointCoord - vec2(0.5)) in float32, per fragment."""
    d = pc.astype(np.float32) - np.float32(0.5)
    return np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(np.float32)


def pbd_inputs() -> dict[str, np.ndarray]:
    """The PBD demo's boxes, from the library's default parameters."""
    from coupledwateranimation_gb300.pbd import pbd_defaults
    return {"pbd_boxes": pbd_boxes(pbd_defaults())}


def sph2d_inputs() -> dict[str, np.ndarray]:
    """The 2D family's inputs, from the library's default parameters (the
    reference app's values)."""
    from coupledwateranimation_gb300.sim2d import defaults2d
    p = defaults2d()
    return {"s2d_state": sph2d_state(p), "s2d_wave": shallow_field(p)}
