"""The CPU restatement of the headless frame (oracle/cwa_render_oracle.cpp),
checked on its own: sprite coverage, empty frames, cube-map face selection."""
from __future__ import annotations

import numpy as np

from coupledwateranimation_gb300 import _abi
from coupledwateranimation_gb300.sim import render_defaults


def _cam_params(w=96, h=64, **kw):
    cam, prm = render_defaults(w, h)
    for k, v in kw.items():
        setattr(prm, k, v)
    return cam, prm


def test_empty_frame_is_clear_colour(lib, orc):
    cam, prm = _cam_params(draw_surface=0, draw_particles=0)
    img = orc.render(np.zeros((0, 4), np.float32), np.zeros((8, 8), np.float32), cam, prm)
    assert img.shape == (64, 96, 4)
    assert (img[..., :3] == 0).all() and (img[..., 3] == 255).all()


def test_isolated_sprite_covers_a_disc(lib, orc):
    # one particle at the look-at point: an 8-pixel sprite keeps pixels with r < 0.5
    # (above y = 0, where the foam mix of particle_fs.glsl keeps it visible)
    cam, prm = _cam_params(draw_surface=0, angle=0.0, particle_scale=1.0)
    cam.center[1] = 0.3
    pos = np.array([[0.0, 0.3, 0.0, 1.0]], np.float32)
    img = orc.render(pos, np.zeros((8, 8), np.float32), cam, prm)
    lit = (img[..., :3] != 0).any(axis=2)
    n = int(lit.sum())
    assert 40 <= n <= 60, n  # ~ pi * 4^2 pixel centres
    ys, xs = np.nonzero(lit)
    assert abs(xs.mean() - 47.5) < 1.0 and abs(ys.mean() - 31.5) < 1.0


def test_skybox_faces_selected_by_major_axis(lib, orc):
    cam, prm = _cam_params(draw_surface=0, draw_particles=0, draw_skybox=1)
    colours = np.array([[255, 0, 0], [0, 255, 0], [0, 0, 255], [255, 255, 0], [0, 255, 255], [255, 0, 255]],
                       np.uint8)
    sky = np.zeros((6, 4, 4, 4), np.uint8)
    sky[..., :3] = colours[:, None, None, :]
    sky[..., 3] = 255
    img = orc.render(np.zeros((0, 4), np.float32), np.zeros((8, 8), np.float32), cam, prm, sky)
    seen = {tuple(c) for c in img[..., :3].reshape(-1, 3)}
    assert seen <= {tuple(c) for c in colours}
    # the view direction (-7, -5, 0) has -x as its major axis: face 1
    assert tuple(img[32, 48, :3]) == tuple(colours[1])


def test_render_structs_defaults(lib):
    cam, prm = render_defaults(320, 200)
    assert list(cam.eye) == [7.0, 4.0, 0.0] and list(cam.center) == [0.0, -1.0, 0.0]
    assert prm.particle_scale == 5.0 and abs(prm.wave_scale - 0.047) < 1e-7 and prm.point_size == 8.0
    assert prm.surface_res == 512 and prm.draw_surface == 1 and prm.draw_particles == 1 and prm.draw_skybox == 0
    assert isinstance(prm, _abi.RenderParams)
