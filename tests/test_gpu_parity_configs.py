"""GPU parity on the benchmark workloads themselves, not only on small scenes.

The sm_103a kernels run through the C ABI on the 32,768-particle / 256^2
workload (C0) and the 1,048,576-particle / 1024^2 workload (C1) at the
bench's sort grid (z cells of h/4, 1,198,563 cells at C1: the 128-tile
look-back chain of the scan, the z-sub-cell windows and the row-mask fill
at full occupancy) and the bench's precision (float32 with cascaded two-sum
neighbour sums), and are checked against the CPU oracle:

  * cell ids, the stable sorted order and the cell starts bit-exact over
    several steps;
  * on the state after 20 steps: rho per particle and pressure / force
    normwise within 1e-5 of the FP64 oracle; integrate and the fixed-point
    deposits bit-exact against the float32 restatement;
  * C0 over its full 200 steps: total mass exact, total energy within 1e-3
    of the FP64 oracle's run, density histograms within 2% (L1);
  * the reference's own scene (20,480 particles, Main.cpp:31) against the
    reference's own O(N^2) loops (rho_pres_comp.glsl:60-68,
    force_comp.glsl:74-88) restated in FP64: the grid path finds the same
    neighbours the all-pairs loop does.
"""
from __future__ import annotations

import numpy as np
import pytest

from _helpers import bits, load_scene, records_f32, rel_inf
from coupledwateranimation_gb300 import PREC_COMPENSATED, Sim, _abi, scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5
ZSUB = 4  # the bench's sort grid: z cells of h / 4


def _workload(config: int):
    return scenes.with_zsub(scenes.CONFIGS[config](), ZSUB).scenes[0]


@pytest.fixture(scope="module")
def c1_scene():
    return _workload(1)


@pytest.fixture(scope="module")
def c0_scene():
    return _workload(0)


def _gpu_cells(g, n: int) -> np.ndarray:
    """Cell id of every particle (upload index) from the GPU's cell starts
    and sorted order."""
    counts = np.diff(g.cell_start)
    cell_of_sorted = np.repeat(np.arange(len(counts), dtype=np.int32), counts)
    out = np.empty(n, np.int32)
    out[g.sorted_id] = cell_of_sorted
    return out


def _grid_steps(orc, sc, steps: int) -> None:
    """The stable sort keeps the order of its input within a cell, and the
    input of step k is the order step k-1 left the particles in: the
    oracle sorts the particles in that order."""
    with Sim(sc.desc, precision=PREC_COMPENSATED) as sim:
        load_scene(sim, 0, sc)
        n = sc.desc.n_particles
        current = np.arange(n, dtype=np.int32)  # upload index of each particle, in the device's order
        for step in range(steps):
            pos = records_f32(sim.download_particles(0))[current, 0:4]
            sim.grid()
            g = sim.download_grid(0)
            start, order, cell_of = orc.grid_build(pos, list(sc.desc.box_lo), orc.cell_edges(sc.desc),
                                                   orc.grid_dims(sc.desc))
            assert np.array_equal(g.cell_start, start), f"cell_start differs at step {step}"
            assert np.array_equal(g.sorted_id, current[order]), f"sorted order differs at step {step}"
            cells = np.empty(n, np.int32)
            cells[current] = cell_of
            assert np.array_equal(_gpu_cells(g, n), cells), f"cell ids differ at step {step}"
            sim.rho_pres()
            sim.force()
            sim.integrate()
            sim.wave()
            sim.synchronize()
            current = g.sorted_id


def test_c0_grid_bit_exact(lib, orc, c0_scene):
    _grid_steps(orc, c0_scene, 4)


def test_c1_grid_bit_exact(lib, orc, c1_scene):
    _grid_steps(orc, c1_scene, 3)


def _one_pass_after(orc, sc, warm_steps: int) -> dict:
    """warm_steps full steps on the GPU, then one pass at a time, each
    checked against the oracle on the state the GPU had before it."""
    out = {}
    with Sim(sc.desc, precision=PREC_COMPENSATED) as sim:
        load_scene(sim, 0, sc)
        sim.step(warm_steps)
        sim.synchronize()
        u_n, u_nm1 = sim.download_wave(0)
        p0 = records_f32(sim.download_particles(0))
        sim.grid()
        sim.rho_pres()
        got = records_f32(sim.download_particles(0))
        ref = orc.to_f64(p0)
        orc.rho_pres(sc.desc, ref, u_n.astype(np.float64))
        out["rho"] = float(np.max(np.abs(got[:, 12] - ref[:, 12]) / np.abs(ref[:, 12])))
        out["p"] = rel_inf(got[:, 13], ref[:, 13])
        sim.force()
        got = records_f32(sim.download_particles(0))
        orc.force(sc.desc, ref, u_n.astype(np.float64))
        out["force"] = [rel_inf(got[:, 8 + c], ref[:, 8 + c]) for c in range(3)]
        # integrate + deposits, bit for bit, on the GPU's own pre-integrate state
        want, want_dep = orc.integrate_f32(sc.desc, got, u_n)
        sim.integrate()
        after = records_f32(sim.download_particles(0))
        dep = sim.download_deposits(0)
        out["integrate_exact"] = bool(np.array_equal(bits(after), bits(want)))
        out["deposits_exact"] = bool(np.array_equal(dep, want_dep))
        out["deposits_nonzero"] = int(np.count_nonzero(want_dep))
        sim.wave()
        new_u, _ = sim.download_wave(0)
        out["wave_exact"] = bool(np.array_equal(bits(new_u), bits(orc.wave_f32(sc.desc, u_n, u_nm1, want_dep))))
    return out


@pytest.mark.parametrize("config", [0, 1])
def test_one_pass_parity_after_20_steps(lib, orc, config, c0_scene, c1_scene):
    sc = c0_scene if config == 0 else c1_scene
    r = _one_pass_after(orc, sc, 20)
    assert r["rho"] <= TOL, f"rho per-particle rel err {r['rho']:.3e}"
    assert r["p"] <= TOL, f"pressure normwise rel err {r['p']:.3e}"
    for c, e in enumerate(r["force"]):
        assert e <= TOL, f"force[{c}] normwise rel err {e:.3e}"
    assert r["integrate_exact"], "integrate differs from the float32 restatement"
    assert r["deposits_exact"], "fixed-point deposits differ"
    assert r["wave_exact"], "wave pass differs from the float32 restatement"


def test_c0_full_run_invariants(lib, orc, c0_scene):
    """C0 over its stated 200 steps (chaotic SPH: judged by invariants)."""
    sc = c0_scene
    steps = 200
    with Sim(sc.desc, precision=PREC_COMPENSATED) as sim:
        load_scene(sim, 0, sc)
        t0 = sim.totals(0)
        sim.step(steps)
        sim.synchronize()
        t1 = sim.totals(0)
        got = records_f32(sim.download_particles(0))
        got_u, _ = sim.download_wave(0)
    n, m = sc.desc.n_particles, sc.desc.mass
    assert t0["mass"] == t1["mass"] == n * np.float64(np.float32(m))
    ref = orc.to_f64(records_f32(sc.particles))
    un = sc.wave.astype(np.float64)
    unm1 = un.copy()
    orc.step(sc.desc, ref, un, unm1, steps)
    tr = orc.totals(sc.desc, ref, un, unm1)
    e_gpu = t1["kinetic"] + t1["potential"]
    e_ref = tr[4] + tr[5]
    assert abs(e_gpu - e_ref) <= 1e-3 * abs(e_ref), (e_gpu, e_ref)
    bins = np.linspace(600, 1400, 81)
    h1, _ = np.histogram(got[:, 12], bins)
    h2, _ = np.histogram(ref[:, 12], bins)
    assert 0.5 * np.abs(h1 - h2).sum() / n <= 0.02
    # The height field is driven by the deposits of particles crossing the
    # surface, so after 200 coupled steps it inherits the trajectories'
    # divergence: judged by its L2 distance and its volume and energy.
    assert np.linalg.norm(got_u - un) / np.linalg.norm(un) <= 1e-3
    for k in ("wave_volume", "wave_energy"):
        want = tr[_abi.TOTALS.index(k)]
        assert abs(t1[k] - want) <= 1e-3 * abs(want), (k, t1[k], want)


def test_reference_scene_matches_all_pairs_loops(lib, orc):
    """The reference's scene, 20,480 particles on its 64 x 5 x 64 cube: the
    grid path's density, pressure and forces equal the reference's O(N^2)
    loops (restated in FP64) within the per-step bar, at the cube's start
    and after 20 steps."""
    sc = scenes.reference()
    assert sc.desc.n_particles == 20480
    with Sim(sc.desc, precision=PREC_COMPENSATED) as sim:
        load_scene(sim, 0, sc)
        for warm in (0, 20):
            if warm:
                sim.step(warm)
                sim.synchronize()
            u_n, _ = sim.download_wave(0)
            p0 = records_f32(sim.download_particles(0))
            sim.grid()
            sim.rho_pres()
            got = records_f32(sim.download_particles(0))
            ref = orc.to_f64(p0)
            orc.rho_pres(sc.desc, ref, u_n.astype(np.float64), brute=True)
            rho_err = np.max(np.abs(got[:, 12] - ref[:, 12]) / np.abs(ref[:, 12]))
            assert rho_err <= TOL, f"step {warm}: rho per-particle rel err {rho_err:.3e}"
            assert rel_inf(got[:, 13], ref[:, 13]) <= TOL
            sim.force()
            got = records_f32(sim.download_particles(0))
            orc.force(sc.desc, ref, u_n.astype(np.float64), brute=True)
            for c in range(3):
                e = rel_inf(got[:, 8 + c], ref[:, 8 + c])
                assert e <= TOL, f"step {warm}: force[{c}] normwise rel err {e:.3e}"
            sim.integrate()
            sim.wave()
            sim.synchronize()
