"""Host-side fault injection on the GPU path (cwa_debug_fail_alloc): every
device allocation of cwa_create, and the wave advance's lazy allocations,
fail cleanly with CWA_ERR_OOM, free what they took, and leave the library
(and an existing sim) usable.  No GPU fault is involved: the failure is
made on the host before the allocation call."""
from __future__ import annotations

import numpy as np
import pytest

from coupledwateranimation_gb300 import CwaError, Sim, _abi

from _helpers import bits, load_scene, small_muller

pytestmark = pytest.mark.gpu
OOM = _abi.CWA_ERR_OOM


@pytest.fixture
def hook(lib):
    f = _abi.load().cwa_debug_fail_alloc
    yield f
    assert f(-1) == 0


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_every_create_allocation_fails_cleanly(hook):
    sc = small_muller((8, 8, 8), 0.03, (96, 80), seed=2)
    with Sim(sc.desc):  # CUDA context and module loading before the baseline
        pass
    free0 = _free_bytes()
    n_fail = 0
    for n in range(200):
        assert hook(n) == 0
        try:
            sim = Sim(sc.desc)
        except CwaError as e:
            assert e.status == OOM and "injected" in str(e)
            n_fail += 1
            continue
        sim.close()  # the countdown now lies past the last allocation
        break
    else:
        pytest.fail("cwa_create made more than 200 allocations")
    assert n_fail >= 20  # every array of the sim went through the hook
    hook(-1)
    assert abs(_free_bytes() - free0) <= 8 << 20  # nothing leaked
    with Sim(sc.desc) as sim:  # and the library still works
        load_scene(sim, 0, sc)
        sim.step(3)
        sim.synchronize()


def test_lazy_wave_allocation_failure_keeps_the_sim(hook):
    sc = small_muller((6, 6, 6), 0.03, (128, 64), seed=4)
    with Sim(sc.desc) as a, Sim(sc.desc) as b:
        for s in (a, b):
            load_scene(s, 0, sc)
            s.step(2)
        hook(0)  # the spare wave buffer of the first blocked advance
        with pytest.raises(CwaError) as ei:
            a.wave_advance(8)
        assert ei.value.status == OOM
        hook(-1)
        a.wave_advance(8)
        for _ in range(8):
            b.wave()
        for s in (a, b):
            s.synchronize()
        wa, wb = a.download_wave(0), b.download_wave(0)
        assert np.array_equal(bits(wa[0]), bits(wb[0])) and np.array_equal(bits(wa[1]), bits(wb[1]))


def test_render_allocation_failures_and_steady_frames(hook):
    # every work-buffer allocation of a first frame (and of the cube map)
    # fails cleanly; a later frame rebuilds what is missing; a frame of an
    # already-seen size allocates nothing
    from coupledwateranimation_gb300.sim import render_defaults

    sc = small_muller((8, 8, 8), 0.03, (64, 64), seed=4)
    sky = np.full((6, 8, 8, 4), 90, np.uint8)
    with Sim(sc.desc) as ref:
        load_scene(ref, 0, sc)
        ref.set_skybox(sky)
        cam, prm = render_defaults(80, 60)
        prm.surface_res = 32
        prm.draw_skybox = 1
        want = ref.render(0, camera=cam, params=prm)
    n_fail = 0
    for n in range(12):
        with Sim(sc.desc) as sim:
            load_scene(sim, 0, sc)
            assert hook(n) == 0
            try:
                sim.set_skybox(sky)
                got = sim.render(0, camera=cam, params=prm)
            except CwaError as e:
                assert e.status == OOM
                n_fail += 1
                assert hook(-1) == 0
                sim.set_skybox(sky)
                got = sim.render(0, camera=cam, params=prm)
            assert hook(-1) == 0
            assert np.array_equal(got, want)
            assert hook(0) == 0  # the next allocation would fail: the same frame needs none
            assert np.array_equal(sim.render(0, camera=cam, params=prm), want)
            assert hook(-1) == 0
    assert n_fail >= 8
