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
    no-allocation scan's check is in test_zz_no_alloc.py).
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
