"""GPU parity tests: the sm_103a kernels, called through the C ABI, against
the CPU oracle on the same seeded inputs.

Bars (written per test):
  * integer work bit-exact: cell ids, stable sorted order, cell start
    arrays, scan outputs, fixed-point deposits;
  * element-wise float32 passes bit-exact against the float32 restatement:
    integrate (+ coupling) and the wave stencil / init;
  * neighbour sums (rho, pressure, force) within 1e-5 relative of the FP64
    oracle (per particle for rho, normwise max|d| / max|ref| otherwise);
  * wave after 1000 steps within 1e-5 relative L2 of the FP64 oracle.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from _helpers import bits, load_scene, records_f32, rel_inf, small_muller, small_reference
from coupledwateranimation_gb300 import PREC_COMPENSATED, PREC_FP32, PREC_FP64, Sim, _abi, scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5


# ------------------------------------------------------------- scan ---------
def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _scan_gpu(lib, x: np.ndarray, inplace=False) -> np.ndarray:
    torch = _torch()
    n = len(x)
    d_in = torch.from_numpy(x.astype(np.int32)).cuda()
    d_out = d_in if inplace else torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.cwa_scan_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.cwa_exclusive_scan_i32(_abi.ptr(d_in), _abi.ptr(d_out), n, _abi.ptr(ws), ws.numel(), stream)
    assert st == 0, _abi.last_error()
    assert lib.cwa_scan_status(n, _abi.ptr(ws), stream) == 0, _abi.last_error()
    torch.cuda.synchronize()
    return d_out[:n].cpu().numpy()


def test_scan_reference_kat(lib, orc):
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).parent / "golden" / "parallel_scan_kat.json").read_text())["cases"]
    for c in cases:
        got = _scan_gpu(lib, np.array(c["input"], np.int32))
        assert got.tolist() == c["exclusive_scan"]


@pytest.mark.parametrize("n", [1, 2, 31, 2047, 2048, 2049, 4096 + 5, 300_763, 1_953_126])
def test_scan_sizes(lib, orc, n):
    x = np.random.default_rng(n).integers(0, 40, n).astype(np.int32)
    assert np.array_equal(_scan_gpu(lib, x), orc.exclusive_scan(x))


def test_scan_in_place(lib, orc):
    x = np.random.default_rng(3).integers(0, 9, 100_001).astype(np.int32)
    assert np.array_equal(_scan_gpu(lib, x, inplace=True), orc.exclusive_scan(x))


# ------------------------------------------------------------- grid ---------
def test_grid_build_operator(lib, orc):
    torch = _torch()
    rng = np.random.default_rng(5)
    n = 200_000
    pos = rng.uniform(-0.05, 1.05, (n, 4)).astype(np.float32)
    pos[::101, 2] = np.float32(0.25)  # points on cell faces
    lo = (C.c_float * 3)(0.0, 0.0, 0.0)
    dims = (C.c_int32 * 3)(40, 30, 50)
    cell = 0.025
    nc = 40 * 30 * 50
    d_pos = torch.from_numpy(pos).cuda()
    d_start = torch.empty(nc + 1, dtype=torch.int32, device="cuda")
    d_idx = torch.empty(n, dtype=torch.int32, device="cuda")
    d_cell = torch.empty(n, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.cwa_grid_workspace_bytes(n, nc), dtype=torch.uint8, device="cuda")
    st = lib.cwa_grid_build(_abi.ptr(d_pos), n, lo, cell, dims, _abi.ptr(d_start), _abi.ptr(d_idx),
                            _abi.ptr(d_cell), _abi.ptr(ws), ws.numel(),
                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, _abi.last_error()
    assert lib.cwa_grid_status(n, nc, _abi.ptr(ws), C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0, \
        _abi.last_error()
    torch.cuda.synchronize()
    start, order, cell_of = orc.grid_build(pos, [0.0, 0.0, 0.0], cell, (40, 30, 50))
    assert np.array_equal(d_cell.cpu().numpy(), cell_of)
    assert np.array_equal(d_start.cpu().numpy(), start)
    assert np.array_equal(d_idx.cpu().numpy(), order)


def _oracle_grid_of(orc, sc_desc, pos_current):
    return orc.grid_build(pos_current, list(sc_desc.box_lo), orc.cell_edges(sc_desc), orc.grid_dims(sc_desc))


@pytest.mark.parametrize("zsub", [1, 4])
def test_sim_grid_bit_exact_across_steps(lib, orc, zsub):
    sc = small_muller((20, 20, 20), 0.02, (64, 64), zsub=zsub)
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        order_ids = np.arange(sc.desc.n_particles, dtype=np.int32)  # current order = upload order
        for step in range(4):
            parts = records_f32(sim.download_particles(0))
            pos_current = parts[order_ids, 0:4]
            sim.grid()
            g = sim.download_grid(0)
            start, order, _ = _oracle_grid_of(orc, sc.desc, pos_current)
            assert np.array_equal(g.cell_start, start), f"cell_start differs at step {step}"
            assert np.array_equal(g.sorted_id, order_ids[order]), f"sorted order differs at step {step}"
            sim.rho_pres()
            sim.force()
            sim.integrate()
            sim.wave()
            sim.synchronize()
            order_ids = g.sorted_id


# ------------------------------------------------- neighbour passes ---------
def _oracle_state(orc, parts_records):
    return orc.to_f64(parts_records)


@pytest.mark.parametrize("preset", ["reference", "muller"])
@pytest.mark.parametrize("prec", [PREC_FP32, PREC_COMPENSATED, PREC_FP64])
@pytest.mark.parametrize("zsub,stage", [(1, 0), (4, 0), (4, -1)])
def test_rho_pres_force_parity(lib, orc, preset, prec, zsub, stage):
    sc = small_reference() if preset == "reference" else small_muller()
    sc.desc.cell_size_z = sc.desc.cell_size / zsub
    with Sim(sc.desc, precision=prec, nb_stage=stage) as sim:
        load_scene(sim, 0, sc)
        u_n, _ = sim.download_wave(0)
        p0 = records_f32(sim.download_particles(0))
        sim.grid()
        sim.rho_pres()
        got = records_f32(sim.download_particles(0))
        ref = orc.to_f64(p0)
        orc.rho_pres(sc.desc, ref, u_n.astype(np.float64))
        rho_err = np.max(np.abs(got[:, 12] - ref[:, 12]) / np.abs(ref[:, 12]))
        assert rho_err <= TOL, f"rho per-particle rel err {rho_err:.3e}"
        assert rel_inf(got[:, 13], ref[:, 13]) <= TOL
        sim.force()
        got = records_f32(sim.download_particles(0))
        orc.force(sc.desc, ref, u_n.astype(np.float64))
        for c in range(3):
            e = rel_inf(got[:, 8 + c], ref[:, 8 + c])
            assert e <= TOL, f"force[{c}] normwise rel err {e:.3e}"


@pytest.mark.parametrize("prec", [PREC_FP32, PREC_COMPENSATED, PREC_FP64])
@pytest.mark.parametrize("zsub,skin", [(1, 0.0), (2, 0.0), (1, 0.2)])
def test_dense_rows_take_the_rescan_path(lib, orc, prec, zsub, skin):
    """h = 4 lattice spacings: a candidate row holds ~128 particles, past the
    64 bits of a row mask, so force rescans those particles' rows (and the
    Verlet density its overflowed lists).  Results still match the oracle."""
    sp = 0.02
    sc = small_muller((14, 14, 14), sp, (32, 32), seed=21, zsub=zsub, skin=skin)
    h = 4.0 * sp
    sc.desc.smoothing_length = h
    sc.desc.cell_size = h * (1.0 + skin) * (1.0 + 1e-6) if skin else h
    sc.desc.cell_size_z = sc.desc.cell_size / zsub
    with Sim(sc.desc, precision=prec, verlet_skin=skin) as sim:
        load_scene(sim, 0, sc)
        u_n, _ = sim.download_wave(0)
        p0 = records_f32(sim.download_particles(0))
        sim.grid()
        sim.rho_pres()
        got = records_f32(sim.download_particles(0))
        ref = orc.to_f64(p0)
        orc.rho_pres(sc.desc, ref, u_n.astype(np.float64))
        rho_err = np.max(np.abs(got[:, 12] - ref[:, 12]) / np.abs(ref[:, 12]))
        assert rho_err <= TOL, f"rho per-particle rel err {rho_err:.3e}"
        sim.force()
        got = records_f32(sim.download_particles(0))
        orc.force(sc.desc, ref, u_n.astype(np.float64))
        for c in range(3):
            e = rel_inf(got[:, 8 + c], ref[:, 8 + c])
            assert e <= TOL, f"force[{c}] normwise rel err {e:.3e}"


# --------------------------------------------- bit-exact element-wise -------
@pytest.mark.parametrize("preset", ["reference", "muller"])
def test_integrate_and_deposits_bit_exact(lib, orc, preset):
    sc = small_reference() if preset == "reference" else small_muller((24, 24, 24), 0.02, (128, 96))
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        for _ in range(3):  # a few steps in, so velocities and the surface are non-trivial
            sim.step(1)
        sim.grid()
        sim.rho_pres()
        sim.force()
        before = records_f32(sim.download_particles(0))
        u_n, u_nm1 = sim.download_wave(0)
        want, want_dep = orc.integrate_f32(sc.desc, before, u_n)
        sim.integrate()
        got = records_f32(sim.download_particles(0))
        assert np.array_equal(bits(got), bits(want)), "integrate differs from the float32 restatement"
        dep = sim.download_deposits(0)
        if preset == "muller":
            assert np.count_nonzero(dep) > 0
            assert np.array_equal(dep, want_dep), "fixed-point deposits differ"
        else:
            assert np.count_nonzero(dep) == 0
        sim.wave()
        new_u, prev_u = sim.download_wave(0)
        assert np.array_equal(bits(prev_u), bits(u_n))
        want_u = orc.wave_f32(sc.desc, u_n, u_nm1, want_dep if preset == "muller" else None)
        assert np.array_equal(bits(new_u), bits(want_u)), "wave step differs from the float32 restatement"
        assert np.count_nonzero(sim.download_deposits(0)) == 0  # the wave pass clears them


@pytest.mark.parametrize("wave", [(37, 29), (64, 20), (4, 3)])
def test_wave_pass_bit_exact_any_width(lib, orc, wave):
    # widths that are not a multiple of 4 take the scalar path of the wave kernel
    sc = small_muller((10, 10, 10), 0.03, wave)
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(2)
        sim.grid()
        sim.rho_pres()
        sim.force()
        sim.integrate()
        dep = sim.download_deposits(0)
        u_n, u_nm1 = sim.download_wave(0)
        sim.wave()
        got, _ = sim.download_wave(0)
    assert np.array_equal(bits(got), bits(orc.wave_f32(sc.desc, u_n, u_nm1, dep)))


@pytest.mark.parametrize("mode", [1.0, 0.0, 0.5])
def test_wave_init_bit_exact(lib, orc, mode):
    sc = small_reference(64)
    sc.desc.wave_mode = mode
    sc.desc.wave_nx, sc.desc.wave_nz = 96, 80
    with Sim(sc.desc) as sim:
        sim.wave_reinit(0)
        a, b = sim.download_wave(0)
    want = orc.wave_init_f32(sc.desc)
    assert np.array_equal(bits(a), bits(want))
    assert np.array_equal(bits(b), bits(want))


def test_wave_1000_steps_l2(lib, orc):
    sc = small_muller((2, 2, 2), 0.02, (256, 256))
    sc.desc.n_particles = 0
    sc.particles = sc.particles[:0]
    with Sim(sc.desc) as sim:
        sim.upload_wave(0, sc.wave, sc.wave)
        for _ in range(1000):
            sim.wave()
        got, _ = sim.download_wave(0)
    a = sc.wave.astype(np.float64)
    b = a.copy()
    for _ in range(1000):
        a, b = orc.wave(sc.desc, a, b), a
    err = np.linalg.norm(got - a) / np.linalg.norm(a)
    assert err <= TOL, f"wave L2 rel err after 1000 steps {err:.3e}"


def test_reference_line_source_mode(lib, orc):
    # mode in (0, 1) switches on the line source of EvolveWave (wave_comp.glsl:177-184)
    sc = small_reference(640)
    sc.desc.wave_mode = 0.5
    with Sim(sc.desc) as sim:
        sim.upload_particles(0, sc.particles)
        sim.wave_reinit(0)
        u0, u1 = sim.download_wave(0)
        sim.wave()
        got, _ = sim.download_wave(0)
    assert np.array_equal(bits(got), bits(orc.wave_f32(sc.desc, u0, u1)))


# ---------------------------------------------------- whole steps -----------
@pytest.mark.parametrize("zsub", [1, 4])
def test_full_step_matches_oracle_one_step(lib, orc, zsub):
    sc = small_muller((20, 20, 20), 0.02, (128, 128), zsub=zsub)
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(1)
        got = records_f32(sim.download_particles(0))
        got_u, _ = sim.download_wave(0)
    ref = orc.to_f64(records_f32(sc.particles))
    un = sc.wave.astype(np.float64)
    unm1 = un.copy()
    orc.step(sc.desc, ref, un, unm1, 1)
    assert np.max(np.abs(got[:, 12] - ref[:, 12]) / ref[:, 12]) <= TOL
    for c in range(3):
        assert rel_inf(got[:, 8 + c], ref[:, 8 + c]) <= TOL
        assert rel_inf(got[:, 4 + c], ref[:, 4 + c]) <= 1e-4  # velocity incl. surface push
    assert rel_inf(got_u, un) <= 1e-5


def test_multistep_invariants(lib, orc):
    """Chaotic SPH: checked through exact mass, energy drift and density histograms."""
    sc = small_muller((16, 16, 16), 0.02, (64, 64))
    steps = 60
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        t0 = sim.totals(0)
        sim.step(steps)
        sim.synchronize()
        t1 = sim.totals(0)
        got = records_f32(sim.download_particles(0))
        got_u, got_um1 = sim.download_wave(0)
    n, m = sc.desc.n_particles, sc.desc.mass
    assert t0["mass"] == t1["mass"] == n * np.float64(np.float32(m))
    ref = orc.to_f64(records_f32(sc.particles))
    un = sc.wave.astype(np.float64)
    unm1 = un.copy()
    orc.step(sc.desc, ref, un, unm1, steps)
    tr = orc.totals(sc.desc, ref, un, unm1)
    e_gpu = t1["kinetic"] + t1["potential"]
    e_ref = tr[4] + tr[5]
    assert abs(e_gpu - e_ref) <= 1e-3 * abs(e_ref)
    bins = np.linspace(600, 1400, 41)
    h1, _ = np.histogram(got[:, 12], bins)
    h2, _ = np.histogram(ref[:, 12], bins)
    assert 0.5 * np.abs(h1 - h2).sum() / n <= 0.02
    assert rel_inf(got_u, un) <= 1e-4


def test_totals_match_oracle(lib, orc):
    sc = small_muller((12, 12, 12), 0.02, (64, 64))
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(5)
        t = sim.totals(0)
        parts = orc.to_f64(records_f32(sim.download_particles(0)))
        a, b = sim.download_wave(0)
    want = orc.totals(sc.desc, parts, a.astype(np.float64), b.astype(np.float64))
    got = np.array([t[k] for k in _abi.TOTALS])
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12)


def test_precision_modes_order(lib, orc):
    sc = small_muller((20, 20, 20), 0.02, (64, 64))
    ref = orc.to_f64(records_f32(sc.particles))
    orc.rho_pres(sc.desc, ref, sc.wave.astype(np.float64))
    errs = {}
    for prec in (PREC_FP32, PREC_COMPENSATED, PREC_FP64):
        with Sim(sc.desc, precision=prec) as sim:
            load_scene(sim, 0, sc)
            sim.grid()
            sim.rho_pres()
            got = records_f32(sim.download_particles(0))
        errs[prec] = np.max(np.abs(got[:, 12] - ref[:, 12]) / ref[:, 12])
    assert errs[PREC_FP64] <= errs[PREC_FP32]
    assert all(e <= TOL for e in errs.values()), errs


# ------------------------------------------------- batching / graphs --------
def _run(scene_list, steps, **kw):
    with Sim([s.desc for s in scene_list], **kw) as sim:
        for k, s in enumerate(scene_list):
            load_scene(sim, k, s)
        sim.step(steps)
        sim.synchronize()
        return [(records_f32(sim.download_particles(k)), sim.download_wave(k)[0]) for k in range(len(scene_list))]


@pytest.mark.parametrize("zsub", [1, 4])
def test_batched_equals_single(lib, zsub):
    scs = [small_muller((10, 12, 14), 0.02, (64, 32), seed=1),
           small_muller((20, 8, 8), 0.03, (48, 48), seed=2),
           scenes.dam_break((9, 9, 9), 0.025, (40, 72), box_hi=(1.5, 1.0, 1.0), seed=3),
           small_muller((7, 9, 11), 0.03, (37, 21), seed=4)]
    for s in scs:
        s.desc.cell_size_z = s.desc.cell_size / zsub
    together = _run(scs, 12)
    for k, s in enumerate(scs):
        alone = _run([s], 12)[0]
        assert np.array_equal(bits(together[k][0]), bits(alone[0])), f"scene {k} particles differ"
        assert np.array_equal(bits(together[k][1]), bits(alone[1])), f"scene {k} wave differs"


def test_work_queue_batch_equals_single(lib):
    """The work-queue form (persistent CTAs taking tiles, largest scenes
    first) over a batch of uneven scenes equals each scene stepped alone."""
    scs = [small_muller((6, 6, 6), 0.03, (32, 32), seed=5),
           small_muller((18, 16, 20), 0.02, (64, 48), seed=6),
           scenes.dam_break((9, 9, 9), 0.025, (40, 72), box_hi=(1.5, 1.0, 1.0), seed=7),
           small_muller((3, 5, 7), 0.03, (21, 37), seed=8)]
    together = _run(scs, 8, nb_queue=1)
    for k, s in enumerate(scs):
        alone = _run([s], 8)[0]
        assert np.array_equal(bits(together[k][0]), bits(alone[0])), f"scene {k} particles differ"
        assert np.array_equal(bits(together[k][1]), bits(alone[1])), f"scene {k} wave differs"


def test_graph_equals_eager(lib):
    sc = small_muller((16, 16, 16), 0.02, (64, 64))
    a = _run([sc], 13, use_graph=True)[0]
    b = _run([sc], 13, use_graph=False)[0]
    assert np.array_equal(bits(a[0]), bits(b[0]))
    assert np.array_equal(bits(a[1]), bits(b[1]))


def test_checkpoint_resume_bit_exact(lib, tmp_path):
    sc = small_muller((16, 16, 16), 0.02, (64, 64))
    full = _run([sc], 20)[0]
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(10)
        sim.save(tmp_path / "ck.bin")
    with Sim(sc.desc) as sim:
        sim.load(tmp_path / "ck.bin")
        assert sim.step_count == 10
        sim.step(10)
        parts = records_f32(sim.download_particles(0))
        u = sim.download_wave(0)[0]
    assert np.array_equal(bits(parts), bits(full[0]))
    assert np.array_equal(bits(u), bits(full[1]))


def test_reference_preset_multistep_runs(lib, orc):
    sc = small_reference(5120)
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(20)
        sim.synchronize()
        got = records_f32(sim.download_particles(0))
    assert np.all(np.isfinite(got))
    assert np.all(got[:, 12] >= sc.desc.rest_rho * 0.1 - 1e-3)


# ------------------------------------------------------ edge cases ----------
def test_edge_cases_grid(lib, orc):
    base = small_muller((4, 4, 4), 0.05, (16, 16))
    cases = {}
    one = base.particles[:1].copy()
    cases["one"] = one
    crowd = np.repeat(base.particles[:1], 500)  # 500 particles in one cell
    crowd["pos"][:, :3] += np.random.default_rng(0).uniform(0, 0.01, (500, 3)).astype(np.float32)
    cases["crowd"] = crowd
    outside = base.particles.copy()
    outside["pos"][::3, 0] = 1.7  # beyond the box: clamped into the last cell
    outside["pos"][1::3, 1] = -0.4
    cases["outside"] = outside
    for name, parts in cases.items():
        d = base.desc.copy()
        d.n_particles = len(parts)
        with Sim(d) as sim:
            sim.upload_particles(0, parts)
            sim.upload_wave(0, base.wave)
            sim.grid()
            g = sim.download_grid(0)
            start, order, _ = _oracle_grid_of(orc, d, records_f32(parts)[:, :4])
            assert np.array_equal(g.cell_start, start), name
            assert np.array_equal(g.sorted_id, order), name
            sim.rho_pres()
            sim.force()
            sim.integrate()
            sim.wave()
            sim.synchronize()


def test_zero_particle_scene_and_mixed_batch(lib):
    a = small_muller((6, 6, 6), 0.05, (32, 32))
    empty = small_muller((2, 2, 2), 0.05, (16, 16))
    empty.desc.n_particles = 0
    empty.particles = empty.particles[:0]
    with Sim([a.desc, empty.desc]) as sim:
        load_scene(sim, 0, a)
        sim.upload_wave(1, empty.wave)
        sim.step(5)
        sim.synchronize()
        assert sim.download_particles(1).shape == (0,)


def test_nonfinite_position_reported(lib):
    sc = small_muller((8, 8, 8), 0.05, (32, 32))
    bad = sc.particles.copy()
    bad["pos"][17, 1] = np.nan
    with Sim(sc.desc) as sim:
        sim.upload_particles(0, bad)
        sim.upload_wave(0, sc.wave)
        sim.grid()
        with pytest.raises(_abi.CwaError) as e:
            sim.synchronize()
        assert e.value.status == _abi.CWA_ERR_NONFINITE
        # the context stays usable
        sim.upload_particles(0, sc.particles)
        sim.step(2)
        sim.synchronize()


def test_invalid_pass_order_rejected(lib):
    sc = small_muller((4, 4, 4), 0.05, (16, 16))
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        with pytest.raises(_abi.CwaError):
            sim.rho_pres()  # no grid pass yet this step
        with pytest.raises(_abi.CwaError):
            sim.upload_particles(0, sc.particles[:10])


def test_full_size_properties(lib):
    """The benchmark's 1,048,576-particle scene: size-independent properties."""
    sc = scenes.config1().scenes[0]
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        t0 = sim.totals(0)
        sim.step(3)
        sim.synchronize()
        g = sim.download_grid(0)
        t1 = sim.totals(0)
        parts = records_f32(sim.download_particles(0))
    n = sc.desc.n_particles
    assert g.cell_start[0] == 0 and g.cell_start[-1] == n
    assert np.all(np.diff(g.cell_start) >= 0)
    assert np.array_equal(np.sort(g.sorted_id), np.arange(n, dtype=np.int32))
    assert t0["mass"] == t1["mass"]
    assert np.all(np.isfinite(parts))


def test_autotune_keeps_state_and_results(lib):
    """The kernel variants change registers, staging and CTA size, never the
    arithmetic order, so a tuned sim steps bit-identically to an untuned one;
    the tuner must also restore the state it trialled on."""
    sc = small_muller((16, 16, 16), 0.02, (64, 64), zsub=2)
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(3)
        before = records_f32(sim.download_particles(0))
        rep = sim.autotune(trial_steps=2)
        assert len(rep["tried"]) == 24 and rep["best_ms"] > 0
        assert np.array_equal(bits(records_f32(sim.download_particles(0))), bits(before))
        assert sim.step_count == 3
        sim.step(5)
        tuned = records_f32(sim.download_particles(0))
        assert sim.options()["nb_scan_minb"] == rep["best"]["nb_scan_minb"]
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(8)
        plain = records_f32(sim.download_particles(0))
    assert np.array_equal(bits(tuned), bits(plain))


@pytest.mark.parametrize("prec", [PREC_FP32, PREC_COMPENSATED])
def test_neighbour_passes_invariant_to_staging_tiles_and_batching(lib, prec):
    """Every particle's neighbour sums run in an order fixed by the particle
    alone, so staging on or off, 64- or 128-particle CTAs, the launch-bound
    variants, the work-queue form of the passes and the scene's place in a batch (here behind a scene
    of odd size) leave every bit unchanged."""
    sc = small_muller((14, 15, 13), 0.02, (48, 40), zsub=4, seed=31)
    odd = small_muller((5, 7, 9), 0.03, (32, 32), seed=32)  # 315 particles: the next scene starts at an odd index
    def run(scene_list, k, **kw):
        with Sim([s.desc for s in scene_list], precision=prec, **kw) as sim:
            for j, s in enumerate(scene_list):
                load_scene(sim, j, s)
            sim.step(6)
            sim.synchronize()
            return records_f32(sim.download_particles(k))
    base = run([sc], 0)
    for kw in ({"nb_stage": -1}, {"nb_threads": 64}, {"nb_threads": 96, "nb_stage": -1}, {"nb_queue": 1},
               {"nb_queue": 1, "nb_threads": 64, "nb_force_minb": 6}, {"nb_force_minb": 8, "nb_scan_minb": 6}):
        assert np.array_equal(bits(run([sc], 0, **kw)), bits(base)), kw
    assert np.array_equal(bits(run([odd, sc], 1)), bits(base)), "batched behind an odd-sized scene"
