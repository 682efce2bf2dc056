"""A mixed workload run by test_gpu_debug_checks.py under both the release
and the index-checked library (chosen by CWA_LIBRARY in the environment):
per-step and Verlet modes, both presets, a batch of scenes with ragged
sizes, every wave-advance variant, the three precisions, a PBD frame and
two rendered frames (tile lists sorted in shared and in global memory).
Prints one digest of every result; a failed device index check surfaces as
CwaError (CWA_ERR_BOUNDS) from a synchronising call and a non-zero exit."""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from coupledwateranimation_gb300 import Sim, _abi  # noqa: E402
from coupledwateranimation_gb300.pbd import PbdSim, make_boxes, pbd_defaults  # noqa: E402

from _helpers import load_scene, small_muller, small_reference  # noqa: E402


def main() -> None:
    h = hashlib.sha256()

    def feed(a):
        h.update(np.ascontiguousarray(a).tobytes())

    scs = [small_muller((10, 9, 11), 0.03, (60, 52), seed=1, zsub=2),
           small_muller((7, 12, 6), 0.03, (128, 40), seed=2),
           small_reference(3000)]
    for prec in (0, 1, 2):
        with Sim([s.desc for s in scs], precision=prec) as sim:
            for k, s in enumerate(scs):
                load_scene(sim, k, s)
            sim.step(12)
            sim.synchronize()
            for k in range(len(scs)):
                feed(sim.download_particles(k))
                feed(sim.download_wave(k)[0])
    verlet = small_muller((10, 10, 10), 0.03, (64, 64), seed=3, skin=0.3)
    with Sim(verlet.desc, verlet_skin=0.3) as sim:
        load_scene(sim, 0, verlet)
        sim.step(15)
        sim.synchronize()
        feed(sim.download_particles(0))
    field = small_muller((6, 6, 6), 0.03, (300, 140), seed=4)
    for v in range(len(_abi.WAVE_BLOCKS)):
        with Sim(field.desc, wave_block=v) as sim:
            load_scene(sim, 0, field)
            sim.step(2)
            sim.wave_advance(16)
            sim.synchronize()
            feed(sim.download_wave(0)[0])
    # headless frames: tiles sorted in shared memory, then a block drawn a
    # few pixels wide, whose tile lists take the radix sort in global scratch
    from coupledwateranimation_gb300.sim import render_defaults
    img = small_muller((16, 16, 16), 0.03, (64, 64), seed=6)
    with Sim(img.desc) as sim:
        load_scene(sim, 0, img)
        sim.step(2)
        sim.set_skybox(np.full((6, 8, 8, 4), 120, np.uint8))
        for scale in (1.5, 0.05):
            cam, prm = render_defaults(130, 97)
            prm.surface_res = 48
            prm.draw_skybox = 1
            prm.particle_scale = scale
            prm.wave_scale = 0.02
            feed(sim.render(0, camera=cam, params=prm))
    p = pbd_defaults()
    p.n_boxes = 512
    with PbdSim(p) as sim:
        sim.upload(make_boxes(p, 7))
        sim.step(3)
        feed(sim.download()["x"])
    print("digest", h.hexdigest())


if __name__ == "__main__":
    main()
