"""cwa_wave_init_from_image (StencilImage2DTripleBuffered::ReinitFromTexture,
StencilImage2DTripleBuffered.cpp:61-77; wave_comp.glsl InitFromImage :76-80)
on the reference's three init textures: bit-exact against the oracle, the
old u^n moved to u^(n-1), other scenes of the sim untouched."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from coupledwateranimation_gb300 import Sim, images

from _helpers import bits, small_reference

pytestmark = pytest.mark.gpu
TEX = np.load(Path(__file__).resolve().parent / "golden" / "init_textures.npz")


@pytest.mark.parametrize("name", ["splash", "wake", "breaking_wave"])
@pytest.mark.parametrize("grid", [(64, 64), (100, 70), (16, 8)])
def test_init_from_image_bit_exact(lib, orc, name, grid):
    sc = small_reference(64)
    sc.desc.wave_nx, sc.desc.wave_nz = grid
    img = images.gl_rows(TEX[name])
    with Sim(sc.desc) as sim:
        sim.wave_reinit(0)
        before, _ = sim.download_wave(0)
        sim.wave_init_from_image(0, img)
        u_n, u_nm1 = sim.download_wave(0)
    assert np.array_equal(bits(u_n), bits(orc.wave_from_image_f32(grid[0], grid[1], img)))
    assert np.array_equal(bits(u_nm1), bits(before))


def test_init_from_image_leaves_other_scenes(lib, orc):
    a, b = small_reference(64), small_reference(64)
    b.desc.wave_nx, b.desc.wave_nz = 48, 40
    with Sim([a.desc, b.desc]) as sim:
        sim.wave_reinit(0)
        sim.wave_reinit(1)
        keep = sim.download_wave(1)
        sim.wave_init_from_image(0, images.gl_rows(TEX["wake"]))
        after = sim.download_wave(1)
        got, _ = sim.download_wave(0)
    assert np.array_equal(bits(keep[0]), bits(after[0])) and np.array_equal(bits(keep[1]), bits(after[1]))
    assert np.array_equal(bits(got), bits(orc.wave_from_image_f32(64, 64, images.gl_rows(TEX["wake"]))))


def test_init_from_image_rejects_bad_input(lib):
    from coupledwateranimation_gb300 import CwaError

    sc = small_reference(64)
    with Sim(sc.desc) as sim:
        with pytest.raises(ValueError):
            sim.wave_init_from_image(0, np.zeros((4, 4, 3), np.uint8))
        with pytest.raises(CwaError):
            sim.wave_init_from_image(3, np.zeros((4, 4, 4), np.uint8))
