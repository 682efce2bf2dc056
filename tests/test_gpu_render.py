"""cwa_render (the reference's display(), Main.cpp:326-474, as CUDA kernels
writing a headless image) against the CPU restatement of the same frame.
Fragment sets, depths and the blend order are exact; shading goes through
the two sides' math libraries, so 8-bit colours may differ by a count or
two after the blends."""
from __future__ import annotations

import numpy as np
import pytest

from coupledwateranimation_gb300 import Sim
from coupledwateranimation_gb300.sim import render_defaults

from _helpers import load_scene, records_f32, small_muller, small_reference

pytestmark = pytest.mark.gpu


def _sky(size=16, seed=3):
    rng = np.random.default_rng(seed)
    base = rng.integers(40, 220, (6, 1, 1, 3))
    ramp = np.linspace(0, 30, size)[None, :, None, None] + np.linspace(0, 20, size)[None, None, :, None]
    sky = np.zeros((6, size, size, 4), np.uint8)
    sky[..., :3] = np.clip(base + ramp, 0, 255).astype(np.uint8)
    sky[..., 3] = 255
    return sky


def _compare(got, want):
    d = np.abs(got.astype(np.int32) - want.astype(np.int32))[..., :3].max(axis=2)
    frac_off = float((d > 2).mean())
    assert frac_off <= 0.002, f"{frac_off:.4%} of pixels differ by more than 2 (max {d.max()})"
    assert float(d.mean()) < 0.1


@pytest.mark.parametrize("case", ["reference", "muller"])
@pytest.mark.parametrize("res,skybox", [(64, 0), (64, 1), (512, 1)])
def test_render_matches_oracle(lib, orc, case, res, skybox):
    sc = small_reference(2048) if case == "reference" else small_muller((12, 12, 12), 0.03, (64, 64))
    sky = _sky()
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(5)
        sim.set_skybox(sky)
        cam, prm = render_defaults(160, 120)
        prm.surface_res = res
        prm.draw_skybox = skybox
        if case == "muller":
            prm.particle_scale = 1.5
            prm.wave_scale = 0.02
        got = sim.render(0, camera=cam, params=prm)
        pos = records_f32(sim.download_particles(0))[:, :4]
        u_n, _ = sim.download_wave(0)
    want = orc.render(pos, u_n, cam, prm, sky)
    assert (got[..., :3] != 0).any()
    _compare(got, want)


def test_render_toggles_and_errors(lib):
    from coupledwateranimation_gb300 import CwaError

    sc = small_reference(512)
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        empty = sim.render(0, 64, 48, draw_surface=0, draw_particles=0)
        assert (empty[..., :3] == 0).all()
        parts = sim.render(0, 64, 48, draw_surface=0)
        assert (parts[..., :3] != 0).any()
        with pytest.raises(CwaError):
            sim.render(0, 64, 48, point_size=0.0)
        with pytest.raises(CwaError):
            sim.render(5, 64, 48)


@pytest.mark.parametrize("point_size", [8.0, 40.0])
def test_render_dense_tiles(lib, orc, point_size):
    # 4096 particles drawn into a few pixels: the tiles under them hold more
    # primitives than a warp sorts in shared memory, so their lists take the
    # radix sort through global scratch; the result must not change
    sc = small_muller((16, 16, 16), 0.03, (64, 64))
    sky = _sky()
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(2)
        sim.set_skybox(sky)
        cam, prm = render_defaults(96, 64)
        prm.surface_res = 64
        prm.draw_skybox = 1
        prm.particle_scale = 0.05
        prm.wave_scale = 0.02
        prm.point_size = point_size
        got = sim.render(0, camera=cam, params=prm)
        pos = records_f32(sim.download_particles(0))[:, :4]
        u_n, _ = sim.download_wave(0)
    want = orc.render(pos, u_n, cam, prm, sky)
    _compare(got, want)
    # the sprites' colour reached the image (not only sky and surface)
    no_particles = orc.render(pos[:0], u_n, cam, prm, sky)
    assert (np.abs(got.astype(np.int32) - no_particles.astype(np.int32)).max(axis=2) > 2).sum() >= 16


@pytest.mark.parametrize("size", [(1, 1), (7, 3), (130, 97), (257, 9)])
def test_render_ragged_image_sizes(lib, orc, size):
    # image edges that cut through 8 x 4 tiles, and images smaller than one tile
    sc = small_reference(2048)
    sky = _sky()
    w, h = size
    with Sim(sc.desc) as sim:
        load_scene(sim, 0, sc)
        sim.step(3)
        sim.set_skybox(sky)
        cam, prm = render_defaults(w, h)
        prm.surface_res = 64
        prm.draw_skybox = 1
        prm.point_size = 3.0 if max(w, h) < 16 else 8.0
        got = sim.render(0, camera=cam, params=prm)
        pos = records_f32(sim.download_particles(0))[:, :4]
        u_n, _ = sim.download_wave(0)
    want = orc.render(pos, u_n, cam, prm, sky)
    assert got.shape == (h, w, 4)
    _compare(got, want)
