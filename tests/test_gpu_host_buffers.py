"""Particle uploads and downloads through page-locked host buffers, as the
benchmark's end-to-end leg uses them: aligned, unaligned and pageable
buffers must give the same sim state and the same host bytes, in upload
order, and a download writes nothing outside the records
(cwa_upload_particles / cwa_download_particles, the SSBO upload of
init_particles, CoupledWaterAnimation/Main.cpp:764-782)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from coupledwateranimation_gb300 import Sim, _abi

from _helpers import small_muller

pytestmark = pytest.mark.gpu


def _pinned(nbytes: int):
    torch = pytest.importorskip("torch")
    buf = torch.empty(nbytes + 64, dtype=torch.uint8, pin_memory=True)
    buf.numpy()[:] = 0
    return buf


@pytest.mark.parametrize("offset", [0, 16, 4])
def test_pinned_and_pageable_routes_agree(lib, offset):
    sc = small_muller((14, 10, 12), 0.03, (96, 64), seed=21)
    n = sc.desc.n_particles
    rec = np.ascontiguousarray(sc.particles).view(np.uint8).reshape(-1)
    buf = _pinned(rec.size)
    view = buf.numpy()[offset:offset + rec.size]
    view[:] = rec
    ptr = buf.data_ptr() + offset
    lib_ = _abi.load()
    sims = [Sim(sc.desc), Sim(sc.desc)]
    try:
        sims[0].upload_particles(0, sc.particles)  # pageable numpy records
        _abi.check(lib_.cwa_upload_particles(sims[1].handle, 0, C.c_void_p(ptr), n), "upload")
        for s in sims:
            s.upload_wave(0, sc.wave, sc.wave)
            s.step(7)
        want = sims[0].download_particles(0).view(np.uint8).reshape(-1)
        view[:] = 0
        _abi.check(lib_.cwa_download_particles(sims[1].handle, 0, C.c_void_p(ptr), n), "download")
        assert np.array_equal(view, want)
        # the other direction: pinned download from the pageable-loaded sim
        view[:] = 0
        _abi.check(lib_.cwa_download_particles(sims[0].handle, 0, C.c_void_p(ptr), n), "download")
        assert np.array_equal(view, want)
        # and the download leaves nothing outside the records
        if offset:
            assert not buf.numpy()[:offset].any()
        assert not buf.numpy()[offset + rec.size:].any()
    finally:
        for s in sims:
            s.close()


def test_pinned_round_trip_is_identity(lib):
    sc = small_muller((9, 9, 9), 0.03, (64, 64), seed=5)
    n = sc.desc.n_particles
    rec = np.ascontiguousarray(sc.particles).view(np.uint8).reshape(-1)
    buf = _pinned(rec.size)
    buf.numpy()[:rec.size] = rec
    lib_ = _abi.load()
    with Sim(sc.desc) as sim:
        _abi.check(lib_.cwa_upload_particles(sim.handle, 0, C.c_void_p(buf.data_ptr()), n), "upload")
        buf.numpy()[:] = 0
        _abi.check(lib_.cwa_download_particles(sim.handle, 0, C.c_void_p(buf.data_ptr()), n), "download")
    assert np.array_equal(buf.numpy()[:rec.size], rec)
