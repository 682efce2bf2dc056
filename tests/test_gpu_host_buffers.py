"""Particle and height-field uploads and downloads through page-locked host
buffers, as the benchmark's end-to-end leg uses them.  Aligned page-locked
buffers are read and written by the library's kernels over the host link;
unaligned and pageable ones go through cudaMemcpyAsync.  All routes must give
the same sim state and the same host bytes, in upload order, and a download
writes nothing outside the records or the field (cwa_upload_particles /
cwa_download_particles, the SSBO upload of init_particles,
CoupledWaterAnimation/Main.cpp:764-782; cwa_upload_wave / cwa_download_wave)."""
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


def _field_ptr(buf, offset):
    return C.c_void_p(buf.data_ptr() + offset)


@pytest.mark.parametrize("wave,offset", [((96, 64), 0), ((65, 63), 0), ((65, 63), 4), ((96, 64), 8)])
def test_wave_fields_through_pinned_buffers(lib, wave, offset):
    """Height fields uploaded and downloaded through page-locked buffers
    (aligned: kernel copies over the host link; unaligned: cudaMemcpyAsync;
    a cell count that is not a multiple of 4 exercises the copy's tail) equal
    the pageable route byte for byte, and write nothing outside the field."""
    sc = small_muller((10, 8, 10), 0.03, wave, seed=33)
    nx, nz = sc.desc.wave_nx, sc.desc.wave_nz
    cells = nx * nz
    u0 = np.ascontiguousarray(sc.wave, np.float32).reshape(-1)
    u1 = (u0 * np.float32(0.75)).astype(np.float32)
    bufs = [_pinned(cells * 4 + 64) for _ in range(2)]
    for b, u in zip(bufs, (u0, u1)):
        b.numpy()[offset:offset + cells * 4] = u.view(np.uint8)
    lib_ = _abi.load()
    sims = [Sim(sc.desc), Sim(sc.desc)]
    try:
        for s in sims:
            s.upload_particles(0, sc.particles)
        sims[0].upload_wave(0, u0.reshape(nz, nx), u1.reshape(nz, nx))
        _abi.check(lib_.cwa_upload_wave(sims[1].handle, 0, _field_ptr(bufs[0], offset), _field_ptr(bufs[1], offset),
                                        nx, nz), "upload_wave")
        for s in sims:
            s.step(5)
        want_n, want_m = sims[0].download_wave(0)
        for b in bufs:
            b.numpy()[:] = 0
        _abi.check(lib_.cwa_download_wave(sims[1].handle, 0, _field_ptr(bufs[0], offset),
                                          _field_ptr(bufs[1], offset), nx, nz), "download_wave")
        for b, want in zip(bufs, (want_n, want_m)):
            got = b.numpy()
            assert np.array_equal(got[offset:offset + cells * 4], want.reshape(-1).view(np.uint8))
            assert not got[:offset].any() and not got[offset + cells * 4:].any()
        # and the particles stepped the same way from both uploads
        assert np.array_equal(sims[0].download_particles(0).view(np.uint8),
                              sims[1].download_particles(0).view(np.uint8))
    finally:
        for s in sims:
            s.close()


def test_pinned_buffers_of_a_later_scene(lib):
    """Pinned uploads and downloads of the second scene of a batch (records
    at a nonzero offset in the sim's arrays) equal the pageable route."""
    a = small_muller((8, 8, 8), 0.03, (64, 64), seed=3)
    b = small_muller((12, 9, 7), 0.03, (72, 40), seed=4)
    n = b.desc.n_particles
    rec = np.ascontiguousarray(b.particles).view(np.uint8).reshape(-1)
    buf = _pinned(rec.size)
    buf.numpy()[:rec.size] = rec
    lib_ = _abi.load()
    sims = [Sim([a.desc, b.desc]), Sim([a.desc, b.desc])]
    try:
        for s in sims:
            s.upload_particles(0, a.particles)
            s.upload_wave(0, a.wave, a.wave)
            s.upload_wave(1, b.wave, b.wave)
        sims[0].upload_particles(1, b.particles)
        _abi.check(lib_.cwa_upload_particles(sims[1].handle, 1, C.c_void_p(buf.data_ptr()), n), "upload")
        for s in sims:
            s.step(4)
        want = sims[0].download_particles(1).view(np.uint8).reshape(-1)
        buf.numpy()[:] = 0
        _abi.check(lib_.cwa_download_particles(sims[1].handle, 1, C.c_void_p(buf.data_ptr()), n), "download")
        assert np.array_equal(buf.numpy()[:rec.size], want)
        assert not buf.numpy()[rec.size:].any()
        assert np.array_equal(sims[0].download_particles(0).view(np.uint8),
                              sims[1].download_particles(0).view(np.uint8))
    finally:
        for s in sims:
            s.close()


def test_buffer_running_past_its_registration(lib):
    """A host buffer whose first pages are page-locked (cudaHostRegister) and
    whose tail is not.  The library checks both ends of the range before its
    kernels touch host memory, so no kernel reads or writes past the
    registration; the copy engine then refuses the mixed range (invalid
    argument), which comes back as CWA_ERR_CUDA, and the sim stays usable:
    the same records through pageable memory step exactly as in a sim that
    never saw the error."""
    torch = pytest.importorskip("torch")
    import os
    cudart = torch.cuda.cudart()
    page = os.sysconf("SC_PAGE_SIZE")
    sc = small_muller((24, 20, 24), 0.02, (64, 64), seed=41)
    n = sc.desc.n_particles
    rec = np.ascontiguousarray(sc.particles).view(np.uint8).reshape(-1)
    raw = np.zeros(rec.size + 2 * page, np.uint8)
    off = (-raw.ctypes.data) % page
    view = raw[off:off + rec.size]
    view[:] = rec
    reg = (rec.size // 2) // page * page  # the first whole pages of the first half
    assert reg > 0
    assert int(cudart.cudaHostRegister(view.ctypes.data, reg, 0)) == 0
    lib_ = _abi.load()
    sims = [Sim(sc.desc), Sim(sc.desc)]
    try:
        for s in sims:
            s.upload_particles(0, sc.particles)
            s.upload_wave(0, sc.wave, sc.wave)
        st = lib_.cwa_upload_particles(sims[1].handle, 0, C.c_void_p(view.ctypes.data), n)
        assert st in (_abi.CWA_OK, _abi.CWA_ERR_CUDA)
        if st != _abi.CWA_OK:
            sims[1].upload_particles(0, sc.particles)  # the next call is not failed by the last error
        st = lib_.cwa_download_particles(sims[1].handle, 0, C.c_void_p(view.ctypes.data), n)
        assert st in (_abi.CWA_OK, _abi.CWA_ERR_CUDA)
        if st == _abi.CWA_OK:
            assert np.array_equal(view, rec)
        for s in sims:
            s.step(3)
        assert np.array_equal(sims[1].download_particles(0).view(np.uint8),
                              sims[0].download_particles(0).view(np.uint8))
    finally:
        for s in sims:
            s.close()
        assert int(cudart.cudaHostUnregister(view.ctypes.data)) == 0
