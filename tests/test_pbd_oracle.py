"""The PBD box collisions' CPU restatement (oracle/cwa_pbd_oracle.cpp) on its own."""
from __future__ import annotations

import numpy as np

from coupledwateranimation_gb300.pbd import make_boxes, pbd_defaults


def test_free_flight_without_contacts(lib, orc):
    p = pbd_defaults()
    p.n_boxes = 2
    p.g[1] = 0.0
    b = make_boxes(p, 1)
    b["x"][0, :3] = (-0.5, 0.0, 0.0)
    b["x"][1, :3] = (0.5, 0.0, 0.0)
    b["v"][:, :3] = (0.1, 0.0, 0.0)
    out = orc.pbd_step(p, b, 1)
    v = np.float32(0.999) * np.float32(0.1)
    assert np.isclose(out["x"][0, 0], -0.5 + 0.02 * v, atol=1e-7)
    assert (out["n"] == 0).all() and (out["color"] == 1).all()


def test_overlapping_pair_separates_symmetrically(lib, orc):
    p = pbd_defaults()
    p.n_boxes = 2
    p.g[1] = 0.0
    b = make_boxes(p, 2)
    b["hw"][:, :3] = 0.05
    b["rm"] = 1.0 / 0.05 ** 3
    b["x"][0, :3] = (-0.04, 0.0, 0.0)
    b["x"][1, :3] = (0.04, 0.0, 0.0)
    b["v"][:] = 0
    out = orc.pbd_step(p, b, 1)
    assert (out["n"] == 1).all() and (out["color"][:, 1] == 0).all()
    assert out["x"][0, 0] < -0.04 and out["x"][1, 0] > 0.04
    assert np.isclose(out["x"][0, 0], -out["x"][1, 0], atol=1e-7)


def test_pile_stays_in_the_extents(lib, orc):
    p = pbd_defaults()
    out = orc.pbd_step(p, make_boxes(p), 30)
    assert np.isfinite(out["x"]).all()
    assert np.abs(out["x"][:, :3]).max() < 1.0
    assert np.array_equal(orc.pbd_step(p, make_boxes(p), 30).view(np.uint8), out.view(np.uint8))
