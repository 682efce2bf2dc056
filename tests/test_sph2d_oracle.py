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
