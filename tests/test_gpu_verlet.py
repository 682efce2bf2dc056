"""Verlet mode: the grid sort and a list of pairs within h (1 + skin) are
kept until some particle has moved skin h / 2.  Every pair with r < h must
still be found, so the physics equals the per-step mode up to summation
order; rebuild-triggering motion, explicit grid passes, graphs and
checkpoints are checked here."""
from __future__ import annotations

import numpy as np
import pytest

from _helpers import bits, load_scene, records_f32, rel_inf, small_muller
from coupledwateranimation_gb300 import Sim

pytestmark = pytest.mark.gpu

TOL = 1e-5
SKIN = 0.25


def _stirred(seed=5, speed=1.5, **kw):
    """A dam-break block with random velocities, so particles leave their skin."""
    sc = small_muller(**kw)
    rng = np.random.default_rng(seed)
    sc.particles["vel"][:, :3] = rng.uniform(-speed, speed, (len(sc.particles), 3)).astype(np.float32)
    return sc


@pytest.mark.parametrize("zsub", [1, 2])
def test_verlet_density_is_complete_after_rebuilds(lib, orc, zsub):
    sc = _stirred(lattice=(16, 16, 16), spacing=0.02, wave=(64, 64), zsub=zsub, skin=SKIN)
    with Sim(sc.desc, verlet_skin=SKIN) as sim:
        load_scene(sim, 0, sc)
        for _ in range(40):
            sim.step(1)
        sim.synchronize()
        rebuilds = sim.rebuild_count
        assert 1 < rebuilds < 40, rebuilds  # some steps reuse the list, some rebuild
        u_n, _ = sim.download_wave(0)
        before = records_f32(sim.download_particles(0))
        # one more density pass on the current (possibly stale-grid) state
        sim.rho_pres()
        got = records_f32(sim.download_particles(0))
    ref = orc.to_f64(before)
    orc.rho_pres(sc.desc, ref, u_n.astype(np.float64))
    err = np.max(np.abs(got[:, 12] - ref[:, 12]) / ref[:, 12])
    assert err <= TOL, f"rho rel err {err:.3e}: a neighbour was missed"
    assert rel_inf(got[:, 13], ref[:, 13]) <= TOL


def test_verlet_matches_per_step_mode(lib):
    sc = small_muller((16, 16, 16), 0.02, (64, 64), skin=SKIN)
    out = []
    for skin in (0.0, SKIN):
        with Sim(sc.desc, verlet_skin=skin) as sim:
            load_scene(sim, 0, sc)
            sim.step(25)
            sim.synchronize()
            out.append(records_f32(sim.download_particles(0)))
    a, b = out
    assert rel_inf(b[:, :3], a[:, :3]) <= 1e-6
    assert rel_inf(b[:, 4:7], a[:, 4:7]) <= 1e-3
    assert rel_inf(b[:, 12], a[:, 12]) <= 1e-5


def test_verlet_explicit_grid_pass_is_bit_exact(lib, orc):
    sc = _stirred(lattice=(12, 12, 12), spacing=0.025, wave=(32, 32), skin=SKIN)
    with Sim(sc.desc, verlet_skin=SKIN) as sim:
        load_scene(sim, 0, sc)
        sim.step(7)
        sim.synchronize()
        parts = records_f32(sim.download_particles(0))
        ids = sim.download_grid(0).sorted_id      # current order = last rebuild's order
        sim.grid()                                # an explicit pass always rebuilds
        g = sim.download_grid(0)
    start, order, _ = orc.grid_build(parts[ids, 0:4], list(sc.desc.box_lo), orc.cell_edges(sc.desc),
                                     orc.grid_dims(sc.desc))
    assert np.array_equal(g.cell_start, start)
    assert np.array_equal(g.sorted_id, ids[order])


def test_verlet_graph_equals_eager_and_resume(lib, tmp_path):
    sc = _stirred(lattice=(12, 12, 12), spacing=0.025, wave=(32, 32), skin=SKIN)
    res = []
    for graph in (True, False):
        with Sim(sc.desc, verlet_skin=SKIN, use_graph=graph) as sim:
            load_scene(sim, 0, sc)
            sim.step(30)
            sim.synchronize()
            res.append((records_f32(sim.download_particles(0)), sim.rebuild_count))
    assert np.array_equal(bits(res[0][0]), bits(res[1][0]))
    assert res[0][1] == res[1][1]
    with Sim(sc.desc, verlet_skin=SKIN) as sim:
        load_scene(sim, 0, sc)
        sim.step(13)
        sim.save(tmp_path / "v.bin")
    with Sim(sc.desc, verlet_skin=SKIN) as sim:
        sim.load(tmp_path / "v.bin")
        sim.step(17)
        resumed = records_f32(sim.download_particles(0))
    assert np.array_equal(bits(resumed), bits(res[0][0]))


def test_verlet_needs_wide_cells(lib):
    sc = small_muller((4, 4, 4), 0.05, (16, 16))  # cell = h
    from coupledwateranimation_gb300 import _abi
    with pytest.raises(_abi.CwaError) as e:
        Sim(sc.desc, verlet_skin=SKIN)
    assert e.value.status == _abi.CWA_ERR_INVALID_ARG
