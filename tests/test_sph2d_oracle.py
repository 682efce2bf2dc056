"""The 2D solver family's CPU restatement (oracle/cwa2d_oracle.cpp) on its own."""
from __future__ import annotations

import numpy as np

from coupledwateranimation_gb300 import _abi
from coupledwateranimation_gb300.sim2d import defaults2d


def test_init_lattice(lib, orc):
    p = defaults2d()
    parts = orc.init_particles_2d(p, _abi.PARTICLE2D_DTYPE)
    pos = parts["pos"]
    assert len(parts) == 4096
    assert (pos[:, 3] == 1.0).all() and (parts["acc"][:, 3] == 1000.0).all()
    assert np.isclose(pos[0, 0], 0.025) and np.isclose(pos[0, 1], 4.8 - 0.375 + 0.025, atol=1e-6)
    assert np.isclose(pos[127, 0], 9.6 * 127 / 128 + 0.025, atol=1e-5)


def test_still_water_stays_still(lib, orc):
    p = defaults2d()
    w = np.zeros((p.wave_cells, 4), np.float32)
    w[:, 0] = 4.8
    a = orc.wave_iter_2d_f32(p, w, 0)
    b = orc.wave_iter_2d_f32(p, a, 1)
    assert np.array_equal(b[:, 0], w[:, 0]) and (b[:, 1] == 0).all()


def test_wave_init_and_splash(lib, orc):
    p = defaults2d()
    w = orc.wave_init_2d_f32(p)
    assert np.isclose(w[64, 0], 4.8 + 0.96 * np.exp(-(64 / 127 - 0.5) ** 2 / 0.005), rtol=1e-6)
    assert np.isclose(w[0, 0], 4.8, atol=1e-6) and w[10, 1] < 0 < w[117, 1]
    s = orc.wave_init_2d_f32(p, w, splash=True)
    assert s[64, 0] < w[64, 0] and np.isclose(s[0, 0], w[0, 0], atol=1e-6)


def test_density_of_the_initial_lattice(lib, orc):
    p = defaults2d()
    parts = orc.init_particles_2d(p, _abi.PARTICLE2D_DTYPE)
    w = orc.wave_init_2d_f32(p)
    out = orc.density_2d(p, parts, w)
    rho = out["acc"][:, 3]
    assert (rho >= 1000.0).all()
    # spacing 0.075 x 0.05625 against 2r = 0.05: the block is sparser than rest, so it clamps
    assert np.isfinite(out["vel"][:, 3]).all()


def _wave1d_numpy(p, cur, prev, mode=None):
    """Wave1D_cs.glsl restated in numpy float32 (one rounding per operation):
    IterateWave when mode is None, else InitWave MODE_INIT_1."""
    f = np.float32
    lam, beta, atten = f(p.wave_lambda), f(p.wave_beta), f(p.wave_atten)
    c0 = cur.astype(f)
    c1 = prev.astype(f)
    e0 = np.vstack([c0[1:], np.zeros((1, 4), f)])
    w0 = np.vstack([np.zeros((1, 4), f), c0[:-1]])
    if mode is None:
        a = (f(2) - f(2) * lam) - beta
        w = atten * ((a * c0 + lam * (e0 + w0)) - (f(1) - beta) * c1)
    else:
        w = c0 - (f(0.5) * lam) * ((e0 - f(2) * c0) + w0)
    w[:, 1] = (w[:, 0] - c1[:, 0]) / f(2)
    w[:, 2] = (w[:, 0] - f(2) * c0[:, 0]) + c1[:, 0]
    out = w.copy()  # FreeBC: the end cells take their inner neighbours' values
    out[0] = w[1]
    out[-1] = w[-2]
    return out


def test_wave1d_matches_numpy_float32(lib, orc):
    from coupledwateranimation_gb300.sim2d import WAVE2D_1D
    p = defaults2d(WAVE2D_1D)
    assert (p.wave_cells, p.wave_substeps, p.wave_kind) == (1024, 10, 1)
    assert np.isclose(p.wave_lambda, 0.01) and np.isclose(p.wave_atten, 0.9995) and np.isclose(p.wave_beta, 0.001)
    g0 = orc.wave1d_init_2d_f32(p, 0)
    cen = int(0.25 * 1024)
    x = cen - np.arange(1024)
    assert np.allclose(g0[:, 0], 0.1 * np.exp(-(x * x) / 5000.0), rtol=1e-5, atol=1e-37)  # float32 argument: |arg| ulps
    assert (g0[:, 1:] == 0).all() and g0[cen, 0] == np.float32(0.1)
    g1 = orc.wave1d_init_2d_f32(p, 1, cur=g0)  # the older field is still zero
    assert np.array_equal(g1.view(np.uint32), _wave1d_numpy(p, g0, np.zeros_like(g0), mode=1).view(np.uint32))
    rng = np.random.default_rng(3)
    cur = rng.standard_normal((1024, 4)).astype(np.float32)
    prev = rng.standard_normal((1024, 4)).astype(np.float32)
    got = orc.wave1d_iter_2d_f32(p, cur, prev)
    assert np.array_equal(got.view(np.uint32), _wave1d_numpy(p, cur, prev).view(np.uint32))


def test_wave1d_bump_spreads_and_decays(lib, orc):
    from coupledwateranimation_gb300.sim2d import WAVE2D_1D
    p = defaults2d(WAVE2D_1D)
    prev = orc.wave1d_init_2d_f32(p, 0)
    cur = orc.wave1d_init_2d_f32(p, 1, cur=prev)
    peak0 = cur[:, 0].max()
    for _ in range(2000):
        cur, prev = orc.wave1d_iter_2d_f32(p, cur, prev), cur
    assert np.isfinite(cur).all()
    assert cur[:, 0].max() < 0.8 * peak0  # attenuation 0.9995 per step
    assert cur[0, 0] == cur[1, 0] and cur[-1, 0] == cur[-2, 0]  # free ends copy their neighbours
