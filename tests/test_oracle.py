"""CPU tests of the oracle: pinned to the reference's scan KAT, cross-checked
against independent numpy restatements, brute-force vs grid neighbour sums,
closed-form wave modes and float32-vs-float64 agreement."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from coupledwateranimation_gb300 import _abi

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_scan_matches_reference_kat(orc):
    # SphWave2D/ParallelScan.cpp:124-155 and UniformGrid2D/ParallelScan.cpp:113-127
    cases = json.loads((GOLDEN / "parallel_scan_kat.json").read_text())["cases"]
    assert len(cases) == 2
    assert cases[0]["input"] == [1, 0, 1, 0, 1, 2, 1, 2, 1, 2, 0, 1, 0, 2, 1, 0]
    for c in cases:
        got = orc.exclusive_scan(np.array(c["input"], np.int32))
        assert got.tolist() == c["exclusive_scan"]


@pytest.mark.parametrize("n", [0, 1, 2, 17, 1000, 4097])
def test_scan_random(orc, n):
    x = np.random.default_rng(n).integers(0, 50, n).astype(np.int32)
    want = np.concatenate([[0], np.cumsum(x)[:-1]]).astype(np.int32) if n else x
    assert np.array_equal(orc.exclusive_scan(x), want)


def _numpy_grid(pos, lo, cell, dims):
    """Independent numpy restatement of the float32 cell hash + stable sort."""
    pos = pos.astype(np.float32)
    t = (pos[:, :3] - np.asarray(lo, np.float32)) / np.float32(cell)
    f = np.floor(t)
    f = np.nan_to_num(f, nan=0.0)
    f = np.clip(f, 0, np.asarray(dims) - 1).astype(np.int64)
    key = (f[:, 0] * dims[1] + f[:, 1]) * dims[2] + f[:, 2]
    order = np.argsort(key, kind="stable")
    counts = np.bincount(key, minlength=int(np.prod(dims)))
    start = np.concatenate([[0], np.cumsum(counts)])
    return start.astype(np.int32), order.astype(np.int32), key.astype(np.int32)


def test_grid_build_matches_numpy(orc):
    rng = np.random.default_rng(1)
    pos = rng.uniform(-0.1, 1.1, (5000, 4)).astype(np.float32)
    pos[::97, 1] = np.float32(0.5)  # exact cell boundaries
    lo, cell, dims = [0.0, 0.0, 0.0], 0.05, (20, 20, 20)
    start, order, cell_of = orc.grid_build(pos, lo, cell, dims)
    s2, o2, k2 = _numpy_grid(pos, lo, cell, dims)
    assert np.array_equal(cell_of, k2)
    assert np.array_equal(start, s2)
    assert np.array_equal(order, o2)


def test_grid_dims_match_library(orc, lib):
    for preset, s in ((0, 0.0), (1, 0.02), (1, 0.0075), (1, 0.004)):
        d = orc.scene_defaults(preset, s, _abi.SceneDesc)
        import ctypes as C
        dims = (C.c_int32 * 3)()
        assert lib.cwa_grid_dims(C.byref(d), dims) == 0
        assert tuple(dims) == orc.grid_dims(d)
    d = orc.scene_defaults(1, 0.0075, _abi.SceneDesc)
    assert orc.grid_dims(d) == (67, 67, 67)
    d = orc.scene_defaults(1, 0.02, _abi.SceneDesc)
    assert orc.grid_dims(d) == (25, 25, 25)


def test_golden_oracle_regression(orc):
    import hashlib
    g = json.loads((GOLDEN / "oracle_regression.json").read_text())
    d = orc.scene_defaults(0, 0.0, _abi.SceneDesc)
    cube = orc.make_reference_cube(d, d.n_particles)
    h = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert h(cube) == g["reference_cube"]["cube_sha256"]
    start, order, _ = orc.grid_build(cube[:, :4], list(d.box_lo), orc.cell_edges(d), orc.grid_dims(d))
    assert h(start) == g["reference_cube"]["cell_start_sha256"]
    assert h(order) == g["reference_cube"]["order_sha256"]
    assert h(orc.wave_init_f32(d)) == g["reference_wave_init"]["sha256"]


def _small_muller(orc, lattice=(8, 8, 8), spacing=0.05, wave=(32, 32), seed=7):
    d = orc.scene_defaults(1, spacing, _abi.SceneDesc)
    orc.scene_set_wave_grid(d, *wave)
    n = int(np.prod(lattice))
    d.n_particles = n
    p = orc.make_dam_break(d, lattice, spacing, 0.05, seed, n)
    u = orc.make_bumps(d, 8, seed + 1, *wave)
    return d, p, u


def test_brute_force_equals_grid_neighbours(orc):
    # The shaders loop over all N (rho_pres_comp.glsl:60-68, force_comp.glsl:74-88);
    # the grid loop must see the same neighbour set.
    for preset in (0, 1):
        if preset == 0:
            d = orc.scene_defaults(0, 0.0, _abi.SceneDesc)
            n = 1280
            p = orc.make_reference_cube(d, n)
            u = orc.wave_init_f32(d)
        else:
            d, p, u = _small_muller(orc)
            n = len(p)
        a = orc.to_f64(p.copy())
        b = a.copy()
        uu = u.astype(np.float64)
        orc.rho_pres(d, a, uu, brute=True)
        orc.rho_pres(d, b, uu, brute=False)
        np.testing.assert_allclose(a[:, 12:14], b[:, 12:14], rtol=1e-12, atol=1e-9)
        orc.force(d, a, uu, brute=True)
        orc.force(d, b, uu, brute=False)
        scale = np.abs(a[:, 8:11]).max()
        assert np.abs(a[:, 8:11] - b[:, 8:11]).max() <= 1e-11 * scale


def test_poly6_self_density(orc):
    # An isolated particle: rho = m * 315 / (64 pi h^9) * h^6 (rho_pres_comp.glsl:66).
    d = orc.scene_defaults(1, 0.02, _abi.SceneDesc)
    d.n_particles = 1
    p = np.zeros((1, 16))
    p[0, :3] = 0.5
    orc.rho_pres(d, p, np.zeros((256, 256)))
    h = d.smoothing_length
    want = d.mass * 315 / (64 * np.pi * h ** 9) * h ** 6
    assert p[0, 12] == pytest.approx(want, rel=1e-12)
    assert p[0, 13] == pytest.approx(d.gas_const * (want - d.rest_rho), rel=1e-12)


def test_wave_standing_mode(orc):
    # Clamped-index (Neumann) borders keep cos(pi k (i+1/2)/N) as an eigenvector of
    # the 5-point Laplacian, so undamped leapfrog evolves it by the 3-term recurrence
    # with growth factor from 2 cos(theta) = 2 - 4 lambda sin^2(pi k / 2N) * 2.
    d = orc.scene_defaults(1, 0.02, _abi.SceneDesc)
    N = 64
    orc.scene_set_wave_grid(d, N, N)
    d.wave_beta = 0.0
    k = 3
    x = np.cos(np.pi * k * (np.arange(N) + 0.5) / N)
    mode = np.outer(np.ones(N), x)
    lam = d.wave_lambda
    mu = -4 * np.sin(np.pi * k / (2 * N)) ** 2  # eigenvalue of the 1D clamped Laplacian
    c = 2 + lam * mu
    a_prev, a_cur = 1.0, 1.0
    u_prev, u_cur = mode.copy(), mode.copy()
    for _ in range(200):
        u_next = orc.wave(d, u_cur, u_prev)
        a_prev, a_cur = a_cur, c * a_cur - a_prev
        u_prev, u_cur = u_cur, u_next
    np.testing.assert_allclose(u_cur, a_cur * mode, atol=1e-9)


def test_wave_f32_tracks_f64(orc):
    d, _, u = _small_muller(orc, wave=(64, 48))
    a64, b64 = u.astype(np.float64), u.astype(np.float64)
    a32, b32 = u.copy(), u.copy()
    for _ in range(300):
        n64 = orc.wave(d, a64, b64)
        n32 = orc.wave_f32(d, a32, b32)
        a64, b64 = n64, a64
        a32, b32 = n32, a32
    err = np.linalg.norm(a32 - a64) / np.linalg.norm(a64)
    assert err < 1e-5


def test_integrate_f32_tracks_f64(orc):
    d, p, u = _small_muller(orc)
    a = orc.to_f64(p.copy())
    orc.rho_pres(d, a, u.astype(np.float64))
    orc.force(d, a, u.astype(np.float64))
    f32 = a.astype(np.float32)
    dep64 = np.zeros((d.wave_nz, d.wave_nx), np.int64)
    b = a.copy()
    orc.integrate(d, b, u.astype(np.float64), dep64)
    out32, dep32 = orc.integrate_f32(d, f32, u)
    np.testing.assert_allclose(out32[:, :3], b[:, :3], rtol=0, atol=1e-6)
    np.testing.assert_allclose(out32[:, 4:7], b[:, 4:7], rtol=1e-4, atol=1e-5)
    # Deposits agree in where they land and (to float rounding) in size.
    assert np.array_equal(dep32 != 0, dep64 != 0)
    np.testing.assert_allclose(dep32.astype(np.float64), dep64.astype(np.float64), rtol=1e-5,
                               atol=2.0 ** 20)


def test_step_conserves_mass_and_moves(orc):
    d, p, u = _small_muller(orc)
    a = orc.to_f64(p.copy())
    un, unm1 = u.astype(np.float64), u.astype(np.float64)
    t0 = orc.totals(d, a, un, unm1)
    orc.step(d, a, un, unm1, 20)
    t1 = orc.totals(d, a, un, unm1)
    assert t1[0] == t0[0]  # mass exact
    assert np.all(np.isfinite(a))
    assert t0[4] == 0.0 and t1[4] > 0.0  # released from rest
    lo, hi = np.array(d.box_lo), np.array(d.box_hi)
    assert np.all(a[:, :3] >= lo - 1e-12) and np.all(a[:, :3] <= hi + 1e-12)


def test_reference_step_runs(orc):
    d = orc.scene_defaults(0, 0.0, _abi.SceneDesc)
    n = 2560
    p = orc.to_f64(orc.make_reference_cube(d, n))
    u = orc.wave_init_f32(d).astype(np.float64)
    un, unm1 = u.copy(), u.copy()
    orc.step(d, p, un, unm1, 3)
    assert np.all(np.isfinite(p))
    assert np.all(p[:, 12] >= d.rest_rho)  # max(resting_rho, rho) (rho_pres_comp.glsl:79)


def test_generators_match_library(orc, lib):
    import ctypes as C
    from coupledwateranimation_gb300 import scenes
    s = scenes.dam_break((10, 12, 14), 0.03, (40, 50), seed=99)
    d = orc.scene_defaults(1, 0.03, _abi.SceneDesc)
    orc.scene_set_wave_grid(d, 40, 50)
    n = 10 * 12 * 14
    d.n_particles = n
    assert bytes(d) == bytes(s.desc)
    p = orc.make_dam_break(d, (10, 12, 14), 0.03, 0.05, 99, n)
    assert np.array_equal(p.view(np.uint32), s.particles.view(np.float32).reshape(-1, 16).view(np.uint32))
    u = orc.make_bumps(d, 8, 99 + scenes.BUMP_SEED, 40, 50)
    assert np.array_equal(u.view(np.uint32), s.wave.view(np.uint32))
    r = scenes.reference()
    dr = orc.scene_defaults(0, 0.0, _abi.SceneDesc)
    assert bytes(dr) == bytes(r.desc)
    cube = orc.make_reference_cube(dr, dr.n_particles)
    assert np.array_equal(cube.view(np.uint32), r.particles.view(np.float32).reshape(-1, 16).view(np.uint32))
    del C


def test_z_subcells_keep_the_neighbour_set(orc):
    # Sorting by finer z cells changes only the search structure.
    d, p, u = _small_muller(orc)
    a = orc.to_f64(p.copy())
    b = a.copy()
    uu = u.astype(np.float64)
    orc.rho_pres(d, a, uu, brute=True)
    d4 = type(d).from_buffer_copy(d)
    d4.cell_size_z = d.cell_size / 4
    orc.rho_pres(d4, b, uu, brute=False)
    np.testing.assert_allclose(a[:, 12:14], b[:, 12:14], rtol=1e-12, atol=1e-9)
    orc.force(d, a, uu, brute=True)
    orc.force(d4, b, uu, brute=False)
    assert np.abs(a[:, 8:11] - b[:, 8:11]).max() <= 1e-11 * np.abs(a[:, 8:11]).max()
    dims = orc.grid_dims(d4)
    assert dims[2] == 4 * orc.grid_dims(d)[2]


def test_oracle_workloads_match_library(orc, lib):
    """The CPU legs of bench.py build their workloads with the oracle's
    generators (oracle/workloads.py); those must be the library's bytes."""
    import ctypes as C
    from coupledwateranimation_gb300 import scenes
    from oracle import workloads
    assert C.sizeof(workloads.SceneDesc) == C.sizeof(_abi.SceneDesc)
    for (a, _), (b, _) in zip(workloads.SceneDesc._fields_, _abi.SceneDesc._fields_):
        assert a == b and getattr(workloads.SceneDesc, a).offset == getattr(_abi.SceneDesc, b).offset
    pairs = [(workloads.config0(), scenes.config0()),
             (workloads.config3(n_scenes=5), scenes.config3(n_scenes=5)),
             (workloads.config4(n_scenes=2), scenes.config4(n_scenes=2))]
    for ow, lw in pairs:
        assert ow.name == lw.name and ow.steps == lw.steps and len(ow.scenes) == len(lw.scenes)
        for o, s in zip(ow.scenes, lw.scenes):
            assert bytes(o.desc) == bytes(s.desc)
            assert np.array_equal(o.particles.view(np.uint32),
                                  s.particles.view(np.float32).reshape(-1, 16).view(np.uint32))
            assert np.array_equal(o.wave.view(np.uint32), s.wave.view(np.uint32))
    r, rl = workloads.reference_preset(), scenes.reference()
    assert bytes(r.desc) == bytes(rl.desc) and r.desc.n_particles == 20480
    assert np.array_equal(r.particles.view(np.uint32), rl.particles.view(np.float32).reshape(-1, 16).view(np.uint32))
