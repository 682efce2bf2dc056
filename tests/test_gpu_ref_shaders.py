"""The sm_103a kernels against the reference's own compute shaders.

tests/golden/ref_shader_outputs.npz holds outputs of
CoupledWaterAnimation/{rho_pres,force,integrate,wave}_comp.glsl compiled as
C++ and run on the CPU (tests/golden/make_ref_shader_golden.py).  The same
seeded inputs (oracle/ref.py) go through the C ABI on the GPU, REFERENCE_3D
preset:
  * rho and pressure within 1e-5 (per particle / normwise) of the FP64
    shader run over all 20,480 particles; force, computed on the GPU's own
    densities, normwise within 1e-5, its w bit-exact;
  * integrate bit-exact against the float32 shader except the surface
    height, which the kernel's bilinear sample rounds differently (a few
    float32 roundings of the field);
  * EvolveWave within two float32 roundings of the field's magnitude (the
    kernels sum the neighbours pairwise, the shader left to right);
  * InitWave and InitFromImage bit-exact;
  * the stand-alone grid build (cwa_grid_build) and the exclusive scan
    (cwa_exclusive_scan_i32) bit-exact against
    UniformGrid2D/ugrid_particles_cs.glsl and prefix_sum_cs.glsl (the
    no-allocation scan's check is in test_zz_no_alloc.py);
  * the 2D family (cwa2d_*): initial particles bit-exact and initial fields
    within 1e-6 (expf), one substep's grid, density and forces within the
    oracle's bars of the double shaders, the shallow-water and Wave1D steps
    bit-exact.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from coupledwateranimation_gb300 import PARTICLE_DTYPE, PREC_COMPENSATED, Sim, _abi, scenes

from _helpers import records_f32

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
G = np.load(GOLDEN / "ref_shader_outputs.npz")
TOL = 1e-5


@pytest.fixture(scope="module")
def x():
    from oracle import ref
    return ref.fixture_inputs(np.load(GOLDEN / "init_textures.npz")["splash"])


def _records(p16: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(p16, np.float32).view(PARTICLE_DTYPE).reshape(-1)


def _desc(n=None, wave=None, mode=None):
    d = scenes.reference().desc
    if n is not None:
        d.n_particles = n
    if wave is not None:
        d.wave_nx, d.wave_nz = wave
    if mode is not None:
        d.wave_mode = mode
    return d


def test_density_and_force_match_the_shaders(lib, x):
    s = G["sph_sample"]
    with Sim(_desc(), precision=PREC_COMPENSATED) as sim:
        sim.upload_particles(0, _records(x["sph"]))
        sim.upload_wave(0, x["sph_wave"], x["sph_wave"])
        sim.grid()
        sim.rho_pres()
        got = records_f32(sim.download_particles(0))
        want = G["rho_f64"]
        assert np.max(np.abs(got[s, 12] - want[:, 0]) / want[:, 0]) <= TOL
        assert np.max(np.abs(got[s, 13] - want[:, 1])) / np.max(np.abs(want[:, 1])) <= TOL
        sim.force()
        got = records_f32(sim.download_particles(0))
    for c in range(3):
        w = G["force_f64"][:, c]
        assert np.max(np.abs(got[s, 8 + c] - w)) / np.max(np.abs(w)) <= TOL, c
    assert np.array_equal(got[s, 11].view(np.uint32), G["force_f32"][:, 3].view(np.uint32))


@pytest.mark.parametrize("mode", [1.0, 0.5])
def test_integrate_matches_the_shader(lib, x, mode):
    with Sim(_desc(n=len(x["integ"]), mode=mode)) as sim:
        sim.upload_particles(0, _records(x["integ"]))
        sim.upload_wave(0, x["sph_wave"], x["sph_wave"])
        sim.integrate()
        got = records_f32(sim.download_particles(0))
    want = G["integ_f32" if mode == 1.0 else "integ_m05_f32"]
    other = [c for c in range(16) if c != 1]
    assert np.array_equal(got[:, other].view(np.uint32), want[:, other].view(np.uint32))
    dy = np.abs(got[:, 1].astype(np.float64) - want[:, 1])
    assert np.count_nonzero(dy) <= len(got) // 20
    assert dy.max() <= 4 * np.finfo(np.float32).eps * np.abs(x["sph_wave"]).max()


@pytest.mark.parametrize("case,size,mode", [("evolve64_m1", "64", 1.0), ("evolve64_m05", "64", 0.5),
                                            ("evolve67_m05", "67", 0.5)])
def test_wave_pass_matches_the_shader(lib, x, case, size, mode):
    un, unm1 = x[f"evolve{size}_un"], x[f"evolve{size}_unm1"]
    with Sim(_desc(wave=(un.shape[1], un.shape[0]), mode=mode)) as sim:
        sim.upload_particles(0, _records(x["sph"]))
        sim.upload_wave(0, un, unm1)
        sim.wave()
        got, prev = sim.download_wave(0)
    want = G[f"{case}_f32"]
    scale = float(np.abs(un).max())
    assert np.abs(got.astype(np.float64) - want).max() <= 2 * np.finfo(np.float32).eps * scale
    assert np.mean(got == want) >= 0.9
    assert np.array_equal(prev, un)  # the rotation: u^(n-1) <- u^n


@pytest.mark.parametrize("case,w,h,mode", [("init64_m1", 64, 64, 1.0), ("init64_m0", 64, 64, 0.0),
                                           ("init64_m05", 64, 64, 0.5), ("init67_m05", 67, 45, 0.5)])
def test_wave_init_matches_the_shader_bit_exactly(lib, case, w, h, mode):
    with Sim(_desc(wave=(w, h), mode=mode)) as sim:
        sim.wave_reinit(0)
        got, _ = sim.download_wave(0)
    assert np.array_equal(got.view(np.uint32), G[f"{case}_f32"].view(np.uint32))


def test_init_from_image_matches_the_shader_bit_exactly(lib):
    tex = np.load(GOLDEN / "init_textures.npz")["splash"]
    with Sim(_desc(wave=(32, 64))) as sim:
        sim.wave_init_from_image(0, tex)
        got, _ = sim.download_wave(0)
    assert np.array_equal(got.view(np.uint32), G["image_f32"].view(np.uint32))


@pytest.mark.parametrize("name", ["grid_a", "grid_b"])
def test_grid_build_matches_the_reference_grid_shader(lib, x, name):
    import torch
    from oracle import ref
    _, lo, hi, cell, dims = ref.GRID_CASES[name]
    pos = x[name]
    n, nc = len(pos), int(np.prod(dims))
    d_pos = torch.from_numpy(pos).cuda()
    d_start = torch.empty(nc + 1, dtype=torch.int32, device="cuda")
    d_idx = torch.empty(n, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.cwa_grid_workspace_bytes(n, nc), dtype=torch.uint8, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.cwa_grid_build(_abi.ptr(d_pos), n, (C.c_float * 3)(*lo), cell, (C.c_int32 * 3)(*dims),
                            _abi.ptr(d_start), _abi.ptr(d_idx), None, _abi.ptr(ws), ws.numel(), stream)
    assert st == 0, _abi.last_error()
    assert lib.cwa_grid_status(n, nc, _abi.ptr(ws), stream) == 0, _abi.last_error()
    start = d_start.cpu().numpy()
    assert np.array_equal(np.diff(start), G[f"{name}_counts"])
    assert np.array_equal(start[:-1], G[f"{name}_offsets"])
    assert np.array_equal(d_idx.cpu().numpy(), G[f"{name}_list"])


@pytest.mark.parametrize("name", ["scan_kat", "scan_1k", "scan_16k"])
def test_exclusive_scan_matches_the_reference_scan_shader(lib, x, name):
    import torch
    xin = torch.from_numpy(x[name]).cuda()
    out = torch.empty_like(xin)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = xin.numel()
    ws = torch.empty(lib.cwa_scan_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    st = lib.cwa_exclusive_scan_i32(_abi.ptr(xin), _abi.ptr(out), n, _abi.ptr(ws), ws.numel(), stream)
    assert st == 0, _abi.last_error()
    assert lib.cwa_scan_status(n, _abi.ptr(ws), stream) == 0, _abi.last_error()
    assert np.array_equal(out.cpu().numpy(), G[f"{name}_out"])


# ---- the 2D family (SphWave2D) ---------------------------------------------
def _sha(a) -> str:
    """SHA-256 of the bytes, NaNs as the positive quiet NaN (the GPU's NaN
    differs from the host's in sign and payload)."""
    import hashlib
    a = np.ascontiguousarray(a).copy()
    if a.dtype.kind == "f":
        a[np.isnan(a)] = np.nan
    return hashlib.sha256(a.tobytes()).hexdigest()


def _f12(rec):
    return np.ascontiguousarray(rec).view(np.float32).reshape(-1, 12)


def test_2d_init_matches_the_shaders(lib):
    """InitParticle (bit-exact) and Shallow1D InitWave and Splash from
    cwa2d_create: the fields go through expf, which the GPU and the host
    library round differently in the last bit, so they are held to 1e-6 of
    the shaders' fields."""
    from coupledwateranimation_gb300.sim2d import Sim2D
    init0, splash = G["s2d_shallow_init"], G["s2d_shallow_splash"]
    with Sim2D() as sim:
        assert _sha(_f12(sim.download_particles())) == str(G["s2d_init_sha"])
        assert np.allclose(sim.download_wave(), init0, rtol=1e-6, atol=1e-6)
        sim.splash()
        assert np.allclose(sim.download_wave(), splash, rtol=1e-6, atol=1e-6)


def test_2d_substep_matches_the_shaders(lib, x):
    """Grid, density, forces on a state with particles past the grid's
    extents and below the floor, against the double shaders: the bars of
    the oracle's own check (rho 1e-5, forces 5e-5 normwise)."""
    from coupledwateranimation_gb300._abi import PARTICLE2D_DTYPE
    from coupledwateranimation_gb300.sim2d import Sim2D
    s = G["s2d_sample"]
    with Sim2D() as sim:
        sim.upload_particles(np.ascontiguousarray(x["s2d_state"]).view(PARTICLE2D_DTYPE).reshape(-1))
        sim.upload_wave(x["s2d_wave"])
        sim.run_pass("grid")
        sim.run_pass("density")
        d = _f12(sim.download_particles()).astype(np.float64)
        sim.run_pass("force")
        f = _f12(sim.download_particles()).astype(np.float64)
    want = G["s2d_density_f64"]
    assert np.array_equal(d[s][:, 3], want[:, 3])
    assert np.max(np.abs(d[s][:, 11] - want[:, 11]) / want[:, 11]) <= 1e-5
    assert np.max(np.abs(d[s][:, 7] - want[:, 7])) / np.max(np.abs(want[:, 7])) <= 2e-5
    assert np.max(np.abs(d[s][:, :2] - want[:, :2])) <= 1e-6
    wf = G["s2d_force_f64"]
    for k in (8, 9):
        assert np.max(np.abs(f[s][:, k] - wf[:, k])) / np.max(np.abs(wf[:, k])) <= 5e-5, k
    for k in (0, 1, 4, 5):
        assert np.max(np.abs(f[s][:, k] - wf[:, k])) / np.max(np.abs(wf[:, k])) <= 1e-5, k


def test_2d_fields_match_the_shaders_bit_exactly(lib):
    """The Lax-Wendroff predictor and corrector on the splash field (the
    predictor's cell 0 aside: two invocations write it, see
    tests/test_ref_shaders.py), and one Wave1D iteration."""
    from coupledwateranimation_gb300._abi import WAVE2D_1D
    from coupledwateranimation_gb300.sim2d import Sim2D, defaults2d
    with Sim2D() as sim:
        sim.upload_wave(G["s2d_shallow_splash"])
        sim.run_pass("wave_predict")
        assert _sha(sim.download_wave()[1:]) == str(G["s2d_shallow_pred_sha"])
        sim.run_pass("wave_correct")
        assert _sha(sim.download_wave()) == str(G["s2d_shallow_corr_sha"])
    with Sim2D(defaults2d(WAVE2D_1D)) as sim:
        sim.upload_wave(G["s2d_wave1d_init1"])
        sim.upload_wave_prev(G["s2d_wave1d_init0"])
        sim.run_pass("wave_iterate")
        assert _sha(sim.download_wave()) == str(G["s2d_wave1d_iter_sha"])


# ---- PBD boxes ---------------------------------------------------------------
def test_pbd_frame_matches_the_shader(lib, x):
    """One frame on the GPU (cwa_pbd_step) against uniform_grid_pbd_3D_cs.glsl
    run on the CPU: the same contacts (every box's constraint count, the
    colours), the continuous fields within the rounding of the shader's
    float atomics (the GPU gathers the contacts in a fixed order)."""
    from coupledwateranimation_gb300._abi import PBD_BOX_DTYPE
    from coupledwateranimation_gb300.pbd import PbdSim, pbd_defaults
    with PbdSim(pbd_defaults()) as sim:
        sim.upload(np.ascontiguousarray(x["pbd_boxes"]).view(PBD_BOX_DTYPE).reshape(-1))
        sim.step(1)
        got = np.ascontiguousarray(sim.download()).view(np.float32).reshape(-1, 32)
    assert _sha(got[:, 29]) == str(G["pbd_counts_sha"]) and _sha(got[:, 0:4]) == str(G["pbd_colors_sha"])
    s = G["pbd_sample"]
    g, w = got[s].astype(np.float64), G["pbd_frame1_f32"].astype(np.float64)
    for sl, tol in ((slice(4, 7), 1e-6), (slice(12, 15), 1e-6), (slice(8, 11), 1e-5),
                    (slice(16, 19), 1e-5), (slice(20, 23), 1e-5)):
        assert np.max(np.abs(g[:, sl] - w[:, sl])) <= tol * np.max(np.abs(w[:, sl])), sl
