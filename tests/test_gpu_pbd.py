"""PBD box collisions on the GPU (cwa_pbd_*, the reference's GridTestPbdGpu3D)
against the float32 CPU restatement: every box field bit for bit, because
both sides accumulate the constraints in the same fixed order."""
from __future__ import annotations

import numpy as np
import pytest

from coupledwateranimation_gb300.pbd import PbdSim, make_boxes, pbd_defaults

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("steps", [1, 5, 40])
def test_pbd_bit_exact(lib, orc, steps):
    p = pbd_defaults()
    boxes = make_boxes(p, 7)
    with PbdSim(p) as sim:
        sim.upload(boxes)
        sim.step(steps)
        got = sim.download()
        pairs = sim.pair_count()
    want = orc.pbd_step(p, boxes, steps)
    assert pairs > 0
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))


def test_pbd_substeps_and_non_cubic_grid(lib, orc):
    p = pbd_defaults()
    p.n_boxes = 3000
    p.grid_cells[0], p.grid_cells[1], p.grid_cells[2] = 12, 16, 20
    p.substeps = 3
    p.extents_lo[1] = -0.8
    boxes = make_boxes(p, 11)
    with PbdSim(p) as sim:
        sim.upload(boxes)
        sim.step(10)
        got = sim.download()
    assert np.array_equal(got.view(np.uint8), orc.pbd_step(p, boxes, 10).view(np.uint8))


def test_pbd_runs_are_deterministic(lib):
    p = pbd_defaults()
    boxes = make_boxes(p, 3)
    outs = []
    for _ in range(2):
        with PbdSim(p) as sim:
            sim.upload(boxes)
            sim.step(25)
            outs.append(sim.download())
    assert np.array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))


def test_pbd_errors(lib):
    from coupledwateranimation_gb300 import CwaError

    p = pbd_defaults()
    with PbdSim(p) as sim:
        with pytest.raises(CwaError):
            sim.step(1)  # nothing uploaded
        with pytest.raises(CwaError):
            sim.upload(make_boxes(p)[:10])
