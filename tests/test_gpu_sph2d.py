"""The 2D solver family (cwa2d_*, the reference's SphWave2D app) on the GPU
against its CPU restatement: the initial lattice and the shallow-water step
bit for bit, each SPH pass from the same input within 1e-5 of FP64, graph
frames equal to eager passes, and the coupled run staying finite."""
from __future__ import annotations

import numpy as np
import pytest

from coupledwateranimation_gb300 import _abi
from coupledwateranimation_gb300.sim2d import Sim2D, defaults2d

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _bits(a):
    """Bit patterns with every NaN canonicalised (the predictor's unused
    half-step value past the last cell is 0/0 on both sides)."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).copy()
    b[np.isnan(np.ascontiguousarray(a, np.float32))] = 0x7FC00000
    return b


def _rel_inf(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    den = np.abs(want).max()
    return float(np.abs(got - want).max() / (den if den > 0 else 1.0))


def test_init_and_wave_step_bit_exact(lib, orc):
    p = defaults2d()
    with Sim2D(p) as sim:
        parts = sim.download_particles()
        w0 = sim.download_wave()
        want = orc.init_particles_2d(p, _abi.PARTICLE2D_DTYPE)
        assert np.array_equal(parts.view(np.uint8), want.view(np.uint8))
        assert np.allclose(w0, orc.wave_init_2d_f32(p), rtol=1e-6, atol=1e-6)
        sim.run_pass("wave_predict")
        a = sim.download_wave()
        sim.run_pass("wave_correct")
        b = sim.download_wave()
    wa = orc.wave_iter_2d_f32(p, w0, 0)
    assert np.array_equal(_bits(a), _bits(wa))
    assert np.array_equal(_bits(b), _bits(orc.wave_iter_2d_f32(p, wa, 1, out_prev=w0)))


def test_wave_after_frames_bit_exact(lib, orc):
    p = defaults2d()
    with Sim2D(p) as sim:
        sim.splash()
        w = sim.download_wave()
        sim.step(25)
        got = sim.download_wave()
    prev = w.copy()
    for _ in range(25):
        a = orc.wave_iter_2d_f32(p, w, 0, out_prev=prev)
        b = orc.wave_iter_2d_f32(p, a, 1, out_prev=w)
        prev, w = a, b
    assert np.array_equal(_bits(got), _bits(w))


@pytest.mark.parametrize("frames", [0, 40])
def test_sph_passes_match_fp64(lib, orc, frames):
    p = defaults2d()
    with Sim2D(p) as sim:
        sim.splash()
        sim.step(frames)
        state = sim.download_particles()
        wave = sim.download_wave()
        sim.run_pass("grid")
        sim.run_pass("density")
        dens = sim.download_particles()
        sim.run_pass("force")
        forc = sim.download_particles()
    want_d = orc.density_2d(p, state, wave)
    assert np.array_equal(dens["pos"][:, 3], want_d["pos"][:, 3])  # enable flags
    assert _rel_inf(dens["pos"][:, :2], want_d["pos"][:, :2]) <= 1e-6
    rho_err = float(np.max(np.abs(dens["acc"][:, 3] - want_d["acc"][:, 3]) / want_d["acc"][:, 3]))
    assert rho_err <= TOL, rho_err
    assert _rel_inf(dens["vel"][:, 3], want_d["vel"][:, 3]) <= TOL  # pressure, normwise
    want_f = orc.force_2d(p, dens, wave, grid_from=state)  # the substep's grid is built before density
    for k in range(2):
        assert _rel_inf(forc["acc"][:, k], want_f["acc"][:, k]) <= TOL, k
        assert _rel_inf(forc["vel"][:, k], want_f["vel"][:, k]) <= TOL, k
    assert _rel_inf(forc["pos"][:, :2], want_f["pos"][:, :2]) <= 1e-6


def test_graph_frames_equal_eager_passes(lib):
    p = defaults2d()
    with Sim2D(p) as a, Sim2D(p) as b:
        a.splash()
        b.splash()
        a.step(6)
        for _ in range(6):
            for _ in range(p.sph_substeps):
                b.run_pass("grid")
                b.run_pass("density")
                b.run_pass("force")
            b.run_pass("wave_predict")
            b.run_pass("wave_correct")
        pa, pb = a.download_particles(), b.download_particles()
        assert np.array_equal(pa.view(np.uint8), pb.view(np.uint8))
        assert np.array_equal(_bits(a.download_wave()), _bits(b.download_wave()))


def test_long_run_stays_finite(lib):
    p = defaults2d()
    with Sim2D(p) as sim:
        sim.splash()
        sim.step(400)
        parts = sim.download_particles()
        w = sim.download_wave()
    assert np.isfinite(parts["pos"]).all() and np.isfinite(parts["vel"]).all()
    assert np.isfinite(w[:, :2]).all()
    assert (parts["pos"][:, 0] > -1).all() and (parts["pos"][:, 0] < 10.6).all()


def test_errors(lib):
    from coupledwateranimation_gb300 import CwaError

    p = defaults2d()
    p.n_particles = 100  # not a multiple of the 128 initial columns
    with pytest.raises(CwaError):
        Sim2D(p)
    with Sim2D(defaults2d()) as sim:
        with pytest.raises(CwaError):
            sim.run_pass("density")  # needs a grid pass first


# ---- the Wave1D kind (Wave1D_cs.glsl, the app's InitWaveEquation) ----

def _w1():
    from coupledwateranimation_gb300.sim2d import WAVE2D_1D
    return defaults2d(WAVE2D_1D)


def test_wave1d_reinit_and_iterate_bit_exact(lib, orc):
    p = _w1()
    with Sim2D(p) as sim:
        newest, older = sim.download_wave(), sim.download_wave_prev()
        # Reinit: MODE_INIT_0 (exp: within float rounding), then MODE_INIT_1
        # on it with a zero older field (bit for bit from the device's bump)
        assert np.allclose(older, orc.wave1d_init_2d_f32(p, 0), rtol=1e-5, atol=1e-37)
        want1 = orc.wave1d_init_2d_f32(p, 1, cur=older, prev=np.zeros_like(older))
        assert np.array_equal(_bits(newest), _bits(want1))
        sim.run_pass("wave_iterate")
        a, a_old = sim.download_wave(), sim.download_wave_prev()
        sim.splash()  # MODE_INIT_1 on the current field
        b, b_old = sim.download_wave(), sim.download_wave_prev()
    assert np.array_equal(_bits(a), _bits(orc.wave1d_iter_2d_f32(p, newest, older)))
    assert np.array_equal(_bits(a_old), _bits(newest))
    assert np.array_equal(_bits(b), _bits(orc.wave1d_init_2d_f32(p, 1, cur=a, prev=a_old)))
    assert np.array_equal(_bits(b_old), _bits(a))


@pytest.mark.parametrize("frames", [1, 5])
def test_wave1d_frames_bit_exact(lib, orc, frames):
    # ten substeps per frame rotate the three buffers by one each frame, so
    # frames replay one graph per buffer phase
    p = _w1()
    rng = np.random.default_rng(frames)
    cur = (0.05 * rng.standard_normal((p.wave_cells, 4))).astype(np.float32)
    old = (0.05 * rng.standard_normal((p.wave_cells, 4))).astype(np.float32)
    with Sim2D(p) as sim:
        sim.upload_wave(cur)
        sim.upload_wave_prev(old)
        sim.step(frames)
        got, got_old = sim.download_wave(), sim.download_wave_prev()
    for _ in range(frames * p.wave_substeps):
        cur, old = orc.wave1d_iter_2d_f32(p, cur, old), cur
    assert np.array_equal(_bits(got), _bits(cur))
    assert np.array_equal(_bits(got_old), _bits(old))


def test_wave1d_graph_frames_equal_eager_passes(lib):
    p = _w1()
    with Sim2D(p) as a, Sim2D(p) as b:
        a.step(4)
        for _ in range(4):
            for _ in range(p.sph_substeps):
                b.run_pass("grid")
                b.run_pass("density")
                b.run_pass("force")
            for _ in range(p.wave_substeps):
                b.run_pass("wave_iterate")
        pa, pb = a.download_particles(), b.download_particles()
        assert np.array_equal(pa.view(np.uint8), pb.view(np.uint8))
        assert np.array_equal(_bits(a.download_wave()), _bits(b.download_wave()))
        assert np.array_equal(_bits(a.download_wave_prev()), _bits(b.download_wave_prev()))


def test_wave_kind_errors(lib):
    from coupledwateranimation_gb300 import CwaError

    p = defaults2d()
    p.wave_kind = 7
    with pytest.raises(CwaError):
        Sim2D(p)
    with Sim2D(defaults2d()) as sim:
        with pytest.raises(CwaError):
            sim.run_pass("wave_iterate")
        with pytest.raises(CwaError):
            sim.download_wave_prev()
    with Sim2D(_w1()) as sim:
        with pytest.raises(CwaError):
            sim.run_pass("wave_predict")
        sim.step(2)
        w = sim.download_wave()
        assert np.isfinite(w).all()
