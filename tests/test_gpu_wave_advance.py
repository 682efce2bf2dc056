"""cwa_wave_advance: the temporally blocked wave stencil (K steps per launch
in 128 x H boxes, TMA-loaded tiles; every (H, K) variant) against single wave
passes and the float32 oracle, bit for bit, and the wave tuner.  The wave
module stepped alone is StencilImage2DTripleBuffered::Compute
(StencilImage2DTripleBuffered.cpp:22-31) over wave_comp.glsl EvolveWave
(:171-206)."""
from __future__ import annotations

import numpy as np
import pytest

from coupledwateranimation_gb300 import Sim
from coupledwateranimation_gb300._abi import WAVE_BLOCKS

from _helpers import bits, load_scene, small_muller, small_reference

pytestmark = pytest.mark.gpu


def _pending_deposits(sim: Sim) -> None:
    """Leave the sim mid-step: integrate has deposited, the wave pass not run."""
    sim.step(2)
    sim.grid()
    sim.rho_pres()
    sim.force()
    sim.integrate()


def _compare(desc_list, load, n, pending=True, **kw):
    sims = [Sim(desc_list, **kw), Sim(desc_list, **kw)]
    try:
        for s in sims:
            load(s)
            if pending:
                _pending_deposits(s)
        sims[0].wave_advance(n)
        for _ in range(n):
            sims[1].wave()
        for s in sims:
            s.synchronize()
        for k in range(len(desc_list)):
            a = sims[0].download_wave(k)
            b = sims[1].download_wave(k)
            assert np.array_equal(bits(a[0]), bits(b[0])), f"scene {k} u^n"
            assert np.array_equal(bits(a[1]), bits(b[1])), f"scene {k} u^(n-1)"
        assert sims[0].step_count == sims[1].step_count
    finally:
        for s in sims:
            s.close()


# widths: multiples of 4 take the TMA path, others the plain-load path;
# sizes span one tile, ragged edges and several tiles in both directions
@pytest.mark.parametrize("wave_block", range(len(WAVE_BLOCKS)))
@pytest.mark.parametrize("wave", [(64, 64), (256, 200), (240, 48), (250, 130), (37, 5), (4, 1), (1, 3)])
@pytest.mark.parametrize("n", [1, 4, 9, 14, 17])
def test_wave_advance_equals_single_passes(lib, wave, n, wave_block):
    sc = small_muller((6, 6, 6), 0.03, wave, seed=5)
    _compare([sc.desc], lambda s: load_scene(s, 0, sc), n, wave_block=wave_block)


@pytest.mark.parametrize("wave_block", range(len(WAVE_BLOCKS)))
def test_wave_advance_batched_mixed_widths(lib, wave_block):
    scs = [small_muller((6, 6, 6), 0.03, w, seed=7 + i) for i, w in enumerate([(128, 96), (130, 77), (512, 24)])]

    def load(s):
        for k, sc in enumerate(scs):
            load_scene(s, k, sc)

    _compare([sc.desc for sc in scs], load, 21, wave_block=wave_block)


@pytest.mark.parametrize("pending", [False, True])
def test_wave_tuner_keeps_state_and_picks_fastest(lib, pending):
    # the tuner restores the wave state (and pending deposits) bit for bit;
    # advancing with the chosen variant then equals single passes
    sc = small_muller((6, 6, 6), 0.03, (500, 300), seed=11)
    sims = [Sim(sc.desc), Sim(sc.desc)]
    try:
        for s in sims:
            load_scene(s, 0, sc)
            if pending:
                _pending_deposits(s)
            else:
                s.step(2)
        before = sims[0].download_wave(0), sims[0].step_count
        rep = sims[0].autotune_wave(12)
        assert rep["steps"] == 16
        ms = rep["ms_per_step"]
        assert set(ms) == set(WAVE_BLOCKS) and all(0 < v < 1e3 for v in ms.values())
        assert ms[rep["best_name"]] == min(ms.values())
        assert sims[0].options()["wave_block"] == rep["best"]
        after = sims[0].download_wave(0), sims[0].step_count
        assert np.array_equal(bits(before[0][0]), bits(after[0][0]))
        assert np.array_equal(bits(before[0][1]), bits(after[0][1]))
        assert before[1] == after[1]
        sims[0].wave_advance(19)
        for _ in range(19):
            sims[1].wave()
        for s in sims:
            s.step(2)
            s.synchronize()
        a, b = sims[0].download_wave(0), sims[1].download_wave(0)
        assert np.array_equal(bits(a[0]), bits(b[0])) and np.array_equal(bits(a[1]), bits(b[1]))
        pa, pb = sims[0].download_particles(0), sims[1].download_particles(0)
        assert np.array_equal(pa.view(np.uint8), pb.view(np.uint8))
    finally:
        for s in sims:
            s.close()


def test_wave_advance_reference_line_source(lib):
    sc = small_reference(640)
    sc.desc.wave_mode = 0.5  # line source on (wave_comp.glsl:177-184)
    sc.desc.wave_nx, sc.desc.wave_nz = 200, 120

    def load(s):
        s.upload_particles(0, sc.particles)
        s.wave_reinit(0)

    _compare([sc.desc], load, 12, pending=False)


@pytest.mark.parametrize("wave_block", range(len(WAVE_BLOCKS)))
@pytest.mark.parametrize("wave_mode", [0.0, 0.5])
def test_wave_advance_uncoupled_interior_boxes(lib, wave_block, wave_mode):
    # an uncoupled scene large enough for interior boxes (no row clamps), with
    # and without the line-source column
    sc = small_reference(640)
    sc.desc.wave_mode = wave_mode
    sc.desc.wave_nx, sc.desc.wave_nz = 760, 300  # wide enough for interior 256-column boxes too

    def load(s):
        s.upload_particles(0, sc.particles)
        s.wave_reinit(0)
        s.wave_advance(3)  # a non-trivial field first (single passes)

    _compare([sc.desc], load, 24, pending=False, wave_block=wave_block)


def test_wave_advance_matches_oracle(lib, orc):
    sc = small_muller((6, 6, 6), 0.03, (248, 100), seed=3)
    sc.desc.n_particles = 0
    sc.particles = sc.particles[:0]
    with Sim(sc.desc) as sim:
        sim.upload_wave(0, sc.wave, sc.wave)
        sim.wave_advance(8)
        got_n, got_nm1 = sim.download_wave(0)
    a = sc.wave.astype(np.float32)
    b = a.copy()
    for _ in range(8):
        a, b = orc.wave_f32(sc.desc, a, b), a
    assert np.array_equal(bits(got_n), bits(a))
    assert np.array_equal(bits(got_nm1), bits(b))


@pytest.mark.parametrize("use_graph", [True, False])
def test_steps_after_wave_advance(lib, use_graph):
    # the buffer renaming invalidates captured graphs; later steps must agree
    sc = small_muller((10, 10, 10), 0.03, (128, 128), seed=9)
    sims = [Sim(sc.desc, use_graph=use_graph), Sim(sc.desc, use_graph=use_graph)]
    try:
        for s in sims:
            load_scene(s, 0, sc)
            s.step(3)
        sims[0].wave_advance(5)
        for _ in range(5):
            sims[1].wave()
        for s in sims:
            s.step(4)
            s.synchronize()
        pa, pb = sims[0].download_particles(0), sims[1].download_particles(0)
        assert np.array_equal(pa.view(np.uint8), pb.view(np.uint8))
        ua, ub = sims[0].download_wave(0), sims[1].download_wave(0)
        assert np.array_equal(bits(ua[0]), bits(ub[0])) and np.array_equal(bits(ua[1]), bits(ub[1]))
    finally:
        for s in sims:
            s.close()


def test_wave_advance_rejects_bad_arguments(lib):
    from coupledwateranimation_gb300 import CwaError

    sc = small_muller((4, 4, 4), 0.03, (64, 64))
    with Sim(sc.desc) as sim:
        with pytest.raises(CwaError):
            sim.wave_advance(-1)
        with pytest.raises(CwaError):
            sim.autotune_wave(0)
        sim.wave_advance(0)
    with pytest.raises(CwaError):
        Sim(sc.desc, wave_block=len(WAVE_BLOCKS))
